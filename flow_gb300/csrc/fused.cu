// fused.cu -- the fused FP64 timestep of the GB300 flow kernel set.
//
// Same scheme, same FP64 arithmetic as the reference timestep
// (omp3/flow.c:10-52), reorganised for GB300, where FP64 issue rate (not
// HBM bandwidth) bounds this code:
//   * no expensive quantity is computed twice: fluxes and velocities are
//     produced once per point and stored; only the 2-flop pressure is
//     recomputed for neighbouring faces;
//   * ghost cells are written by the kernel that produces the interior value
//     (mirror_store), replacing the 19 ghost-fill launches per step;
//   * comparisons, selections and minmod run on the integer pipes
//     (fused_math.cuh), divisions by the mesh spacing become multiplications
//     by per-column / per-row reciprocals, data divisions use a MUFU-seeded
//     reciprocal, and a*b+c contracts into FMA;
//   * the CFL minimum and the dt/dt_h update stay on the device
//     (reduce_array[0..1]) for the advection phase; the host reads the pair
//     once, at the end of the step.
// Results agree with the reference to ~1e-13 relative per cell (tests hold
// them to 1e-12); the bit-exact form is stages.cu.
//
// Every kernel is a column strip: 128 threads own 128 consecutive columns and
// march kRows rows, carrying the values of previous rows in registers.
#include "../../include/flow_gb300.h"
#include "common.cuh"
#include "fused.h"
#include "fused_math.cuh"
#include "profile.h"

namespace flow {
namespace {

constexpr int kCols = 128;
constexpr int kRows = 16;
constexpr double kG1 = kGam - 1.0;

// Extra reduce_array slot used by the fused CFL minimum (uint64 bits of the
// running minimum; all candidates are non-negative, so bit order = value
// order).
constexpr int kRaMinBits = 6;

struct StepArgs {
  int nx, ny, pad;
  const double* edgedx;
  const double* edgedy;
  const double* celldx;
  const double* celldy;
  double* P;
  double* rho;
  double* rho_old;
  double* e;
  double* u;
  double* v;
  double* rho_u;
  double* rho_v;
  double* Qxx;
  double* Qyy;
  double* F_x;
  double* F_y;
  double* uF_x;
  double* uF_y;
  double* vF_x;
  double* vF_y;
  double* ra;
  double dt, dt_h, max_dt;  // Lagrangian-phase pair (host values), max_dt
  int first_step;
};

// ===========================================================================
// Lagrangian phase.

// Pressure (EOS on the fly) -> face momenta -> velocities.  Covers every cell
// (P and rho_old are written for ghosts too, as equation_of_state and the
// rho_old copy of the reference do) and every interior x/y face.  The
// reciprocal of each face density is kept in F_x/F_y (free until the
// advection phase) for the viscous update.  omp3/flow.c:55-70, 110-158.
__global__ void __launch_bounds__(kCols) k_lag_pressure(const StepArgs a) {
  __shared__ double sP[kCols + 1], sR[kCols + 1];
  __shared__ double s_iey[kRows], s_wy0[kRows], s_wy1[kRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const int jj = blockIdx.x * kCols + t;
  const int i0 = blockIdx.y * kRows;
  if (t < kRows) {
    const int ii = i0 + t;
    if (ii >= 1 && ii < ny) {
      const double ey = a.edgedy[ii];
      s_iey[t] = 1.0 / ey;
      s_wy0[t] = a.celldy[ii] / (2.0 * ey);
      s_wy1[t] = a.celldy[ii - 1] / (2.0 * ey);
    }
  }
  double iex = 0.0, wx0 = 0.0, wx1 = 0.0;
  if (jj >= 1 && jj < nx) {
    const double ex = a.edgedx[jj];
    iex = 1.0 / ex;
    wx0 = a.celldx[jj] / (2.0 * ex);
    wx1 = a.celldx[jj - 1] / (2.0 * ex);
  }
  const double dt = a.dt;
  double P_dn = 0.0, r_dn = 0.0;  // cell (ii-1, jj)
  if (i0 >= 1 && jj < nx) {
    const size_t c = cidx(nx, i0 - 1, jj);
    r_dn = a.rho[c];
    P_dn = kG1 * r_dn * a.e[c];
  }
  __syncthreads();
  for (int k = 0; k < kRows; ++k) {
    const int ii = i0 + k;
    if (ii >= ny) break;
    double Pc = 0.0, rc = 0.0;
    if (jj < nx) {
      const size_t c = cidx(nx, ii, jj);
      rc = a.rho[c];
      Pc = kG1 * rc * a.e[c];
      a.P[c] = Pc;
      a.rho_old[c] = rc;
    }
    sP[t + 1] = Pc;
    sR[t + 1] = rc;
    if (t == 0) {
      double Pl = 0.0, rl = 0.0;
      if (jj >= 1 && jj - 1 < nx) {
        const size_t c = cidx(nx, ii, jj - 1);
        rl = a.rho[c];
        Pl = kG1 * rl * a.e[c];
      }
      sP[0] = Pl;
      sR[0] = rl;
    }
    __syncthreads();
    if (ii >= pad && ii < ny - pad && jj >= pad && jj < nx + 1 - pad) {
      const size_t f = fidx(nx, ii, jj);
      const double mom = fma(-(dt * (Pc - sP[t])), iex, a.rho_u[f]);
      const double rbar = fma(rc, wx0, sR[t] * wx1);
      const bool z = d_is_zero(rbar);
      const double inv = z ? 0.0 : d_rcp(rbar);
      const double vel = z ? 0.0 : mom * inv;
      a.rho_u[f] = mom;
      a.u[f] = vel;
      a.F_x[f] = inv;
      mirror_store(a.u, nx + 1, ny, pad, ii, jj, vel, true, false);
    }
    if (ii >= pad && ii < ny + 1 - pad && jj >= pad && jj < nx - pad) {
      const size_t c = cidx(nx, ii, jj);
      const double mom = fma(-(dt * (Pc - P_dn)), s_iey[k], a.rho_v[c]);
      const double rbar = fma(rc, s_wy0[k], r_dn * s_wy1[k]);
      const bool z = d_is_zero(rbar);
      const double inv = z ? 0.0 : d_rcp(rbar);
      const double vel = z ? 0.0 : mom * inv;
      a.rho_v[c] = mom;
      a.v[c] = vel;
      a.F_y[c] = inv;
      mirror_store(a.v, nx, ny + 1, pad, ii, jj, vel, false, true);
    }
    P_dn = Pc;
    r_dn = rc;
    __syncthreads();
  }
}

// Artificial viscous stresses on interior cells, omp3/flow.c:173-207.
__device__ __forceinline__ double visc_stress(double crho, double lo,
                                              double mid, double hi,
                                              double hi2) {
  const double m0 = d_min0(mid - lo);
  const double m1 = d_min0(hi - mid);
  const double m2 = d_min0(hi2 - hi);
  return crho * m1 * (0.5 * (d_abs(m2 - m1) + d_abs(m1 - m0)));
}

__global__ void __launch_bounds__(kCols) k_lag_viscosity(const StepArgs a) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (jj >= nx - pad) return;
  const int i1 = min(i0 + kRows, ny - pad);
  double vm = a.v[cidx(nx, i0 - 1, jj)];
  double v0 = a.v[cidx(nx, i0, jj)];
  double vp = a.v[cidx(nx, i0 + 1, jj)];
  for (int ii = i0; ii < i1; ++ii) {
    const double vp2 = a.v[cidx(nx, ii + 2, jj)];
    const size_t f = fidx(nx, ii, jj);
    const size_t c = cidx(nx, ii, jj);
    const double crho = -kCQ * a.rho[c];
    const double qx = visc_stress(crho, a.u[f - 1], a.u[f], a.u[f + 1], a.u[f + 2]);
    const double qy = visc_stress(crho, vm, v0, vp, vp2);
    a.Qxx[c] = qx;
    a.Qyy[c] = qy;
    mirror_store(a.Qxx, nx, ny, pad, ii, jj, qx, false, false);
    mirror_store(a.Qyy, nx, ny, pad, ii, jj, qy, false, false);
    vm = v0;
    v0 = vp;
    vp = vp2;
  }
}

// Viscous acceleration of the face momenta and velocities,
// omp3/flow.c:212-244.  The face-density reciprocals come from F_x/F_y.
__global__ void __launch_bounds__(kCols) k_lag_viscous_accel(const StepArgs a) {
  __shared__ double s_icy[kRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (threadIdx.x < kRows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) s_icy[threadIdx.x] = 1.0 / a.celldy[ii];
  }
  __syncthreads();
  if (jj >= nx + 1 - pad) return;
  const double icx = 1.0 / a.celldx[jj];
  const double dt = a.dt;
  const int i1 = min(i0 + kRows, ny + 1 - pad);
  double qy_dn = (jj < nx - pad) ? a.Qyy[cidx(nx, i0 - 1, jj)] : 0.0;
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    if (ii < ny - pad) {
      const size_t f = fidx(nx, ii, jj);
      const size_t c = cidx(nx, ii, jj);
      const double mom = fma(-(dt * (a.Qxx[c] - a.Qxx[c - 1])), icx, a.rho_u[f]);
      const double inv = a.F_x[f];
      const double vel = d_is_zero(inv) ? 0.0 : mom * inv;
      a.rho_u[f] = mom;
      a.u[f] = vel;
      mirror_store(a.u, nx + 1, ny, pad, ii, jj, vel, true, false);
    }
    if (jj < nx - pad) {
      const size_t c = cidx(nx, ii, jj);
      const double qy = a.Qyy[c];
      const double mom = fma(-(dt * (qy - qy_dn)), s_icy[k], a.rho_v[c]);
      const double inv = a.F_y[c];
      const double vel = d_is_zero(inv) ? 0.0 : mom * inv;
      a.rho_v[c] = mom;
      a.v[c] = vel;
      mirror_store(a.v, nx, ny + 1, pad, ii, jj, vel, false, true);
      qy_dn = qy;
    }
  }
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
// block; the last block to finish applies the leapfrog dt/dt_h rule and
// writes the pair to reduce_array[0..1].
__global__ void __launch_bounds__(kCols) k_lag_energy_dt(const StepArgs a) {
  __shared__ double s_icy[kRows], s_cy[kRows];
  __shared__ unsigned long long s_warp[kCols / 32];
  __shared__ bool s_last;
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (threadIdx.x < kRows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      s_cy[threadIdx.x] = a.celldy[ii];
      s_icy[threadIdx.x] = 1.0 / a.celldy[ii];
    }
  }
  __syncthreads();
  unsigned long long best = ~0ull;
  const bool col_ok = jj < nx - pad;
  if (col_ok) {
    const double cx = a.celldx[jj];
    const double icx = 1.0 / cx;
    const double dt_h = a.dt_h;
    const int i1 = min(i0 + kRows, ny - pad);
    double v0 = a.v[cidx(nx, i0, jj)];
    for (int ii = i0; ii < i1; ++ii) {
      const int k = ii - i0;
      const size_t c = cidx(nx, ii, jj);
      const size_t f = fidx(nx, ii, jj);
      const double v1 = a.v[c + nx];
      const double r = a.rho[c];
      const double p = a.P[c];
      const double qx = a.Qxx[c], qy = a.Qyy[c];
      const bool rz = d_is_zero(r);
      const double inv_r = rz ? 0.0 : d_rcp(r);
      const double dudx = (a.u[f + 1] - a.u[f]) * icx;
      const double dvdy = (v1 - v0) * s_icy[k];
      const double div_dt = (dudx + dvdy) * dt_h;
      const double e_q = fma(-(dt_h * fma(qx, dudx, qy * dvdy)), inv_r, a.e[c]);
      const double rho_c = r * d_rcp(1.0 + div_dt);
      const double e_c = fma(-(p * div_dt), inv_r, e_q);
      const double work = (0.5 * div_dt) * fma(kG1 * e_c, rho_c, p) * inv_r;
      const double e_new = rz ? 0.0 : e_q - work;
      a.e[c] = e_new;
      mirror_store(a.e, nx, ny, pad, ii, jj, e_new, false, false);
      // CFL: celldx / sqrt(c_s^2 + 2 Q / rho) with c_s^2 = gamma (gamma-1) e.
      const double s2 = (kGam * (kGam - 1.0)) * e_new;
      const double two_inv_r = inv_r + inv_r;
      const double dtx = cx * d_rsqrt(fma(qx, two_inv_r, s2));
      const double dty = s_cy[k] * d_rsqrt(fma(qy, two_inv_r, s2));
      const unsigned long long m = (unsigned long long)dbits(d_min_pos(dtx, dty));
      best = (m < best) ? m : best;
      v0 = v1;
    }
  }
  best = warp_min_u64(best);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = s_warp[0];
    for (int w = 1; w < kCols / 32; ++w) b = (s_warp[w] < b) ? s_warp[w] : b;
    unsigned long long* gmin = reinterpret_cast<unsigned long long*>(a.ra + kRaMinBits);
    atomicMin(gmin, b);
    __threadfence();
    unsigned long long* ticket = reinterpret_cast<unsigned long long*>(a.ra + kRaTicket);
    s_last = (atomicAdd(ticket, 1ull) == (unsigned long long)gridDim.x * gridDim.y - 1);
  }
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    const unsigned long long g =
        atomicAdd(reinterpret_cast<unsigned long long*>(a.ra + kRaMinBits), 0ull);
    const double cfl = d_min_pos(a.max_dt, dfrom((long long)g));
    // Leapfrog rule of omp3/flow.c:103-105, evaluated without contraction.
    const double limited = dmin(cfl, __dmul_rn(FLOW_C_M, a.dt_h));
    const double dt = __dmul_rn(0.5, __dadd_rn(__dmul_rn(kCT, limited), a.dt_h));
    a.ra[kRaDt] = dt;
    a.ra[kRaDtH] = a.first_step ? dt : __dmul_rn(kCT, limited);
    *reinterpret_cast<unsigned long long*>(a.ra + kRaTicket) = 0ull;
    *reinterpret_cast<unsigned long long*>(a.ra + kRaMinBits) = ~0ull;
  }
}

// ===========================================================================
// Advection of mass and energy (omp3/flow.c:293-554).

// Second-order upwind interpolation with the MC-limited slope, for the branch
// already chosen by the wind sign: pos selects the left reconstruction
// base + 0.5*m*(h - w*dt_h), otherwise base - 0.5*m*(h + w*dt_h).
__device__ __forceinline__ double mc_face(bool pos, double da, double db,
                                          double dc, double half_inv,
                                          double two_inv, double base,
                                          double h, double wdt) {
  const double mm = d_minmod(d_minmod(half_inv * da, two_inv * db), two_inv * dc);
  const double w = h + (pos ? -wdt : wdt);
  const double hm = pos ? 0.5 * mm : -0.5 * mm;
  return fma(hm, w, base);
}

// Mass and energy flux through one face.  The four cells straddle the face
// (m2, m1 | p0, p1), vm/v0/vp are the face velocities around it, h_m/h_p the
// cell widths on each side, area the face length, inv_h the reciprocal of the
// face spacing and icd the reciprocal of the downstream cell width.  kSideV0:
// take the Van Leer smoothness side from v0 (the y sweep, omp3/flow.c:477)
// instead of the half-step velocity.
template <bool kSideV0>
__device__ __forceinline__ void mass_energy_flux(
    double vm, double v0, double vp, double rm2, double rm1, double r0,
    double rp1, double em2, double em1, double e0, double ep1, double inv_h,
    double h_m, double h_p, double icd, double area, double dt, double dt_h,
    double* F_out, double* eF_out) {
  const double half_inv = 0.5 * inv_h, two_inv = 2.0 * inv_h;
  const double mm = d_minmod(half_inv * (vp - vm),
                             d_minmod(two_inv * (v0 - vm), two_inv * (vp - v0)));
  const double w_tc = fma(-(0.5 * v0 * dt), mm, v0);
  const double jump = r0 - rm1;
  double lim = 0.0;
  if (!d_is_zero(jump)) {
    const bool up = kSideV0 ? d_ge0(v0) : d_ge0(w_tc);
    const double num = up ? (rm1 - rm2) : (rp1 - r0);
    // Van Leer: (s+|s|)/(1+|s|) with s = num/jump, i.e. 2 num/(jump+num)
    // when num and jump share a sign, else 0.
    if (((dbits(num) ^ dbits(jump)) >= 0) && !d_is_zero(num)) {
      lim = (num + num) * d_rcp(jump + num);
    }
  }
  const bool wpos_ge = d_ge0(w_tc);
  const double rho_up = wpos_ge ? rm1 : r0;
  const double wdt = w_tc * dt_h;
  const double flux =
      fma(w_tc, rho_up,
          (0.5 * d_abs(w_tc)) * (1.0 - d_abs(wdt * icd)) * lim * jump);
  const bool pos = d_gt0(w_tc);
  const double e_face = mc_face(pos, pos ? e0 - em2 : ep1 - em1,
                                pos ? em1 - em2 : e0 - em1,
                                pos ? e0 - em1 : ep1 - e0, half_inv, two_inv,
                                pos ? em1 : e0, pos ? h_m : h_p, wdt);
  *F_out = flux;
  *eF_out = area * e_face * flux;
}

// Conservative update of one cell from its two face fluxes.
template <bool kFirst>
__device__ __forceinline__ void mass_energy_update(
    double r_in, double e_in, double r_old, double coef, double a0, double a1,
    double F0, double F1, double eF0, double eF1, double* r_out,
    double* e_out) {
  const double r_new = fma(-coef, fma(a1, F1, -(a0 * F0)), r_in);
  const double rho_e = fma(-coef, eF1 - eF0, r_old * e_in);
  const double den = kFirst ? r_old : r_new;
  *r_out = r_new;
  *e_out = d_is_zero(den) ? 0.0 : rho_e * d_rcp(den);
}

struct SweepArgs {
  const double* r_in;
  const double* e_in;
  double* r_out;
  double* e_out;
};

// x sweep: CTAs own 127 cells and compute the 128 faces around them (the last
// face is shared with the next CTA and written only by its owner).
template <bool kFirst>
__global__ void __launch_bounds__(kCols) k_mass_sweep_x(const StepArgs a,
                                                        const SweepArgs s) {
  __shared__ double sF[kCols], seF[kCols];
  __shared__ double s_coef[kRows], s_ey0[kRows], s_ey1[kRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int t = threadIdx.x;
  const int jj = pad + blockIdx.x * (kCols - 1) + t;  // face (and cell) column
  const int i0 = pad + blockIdx.y * kRows;
  const double dt = a.ra[kRaDt], dt_h = a.ra[kRaDtH];
  if (t < kRows) {
    const int ii = i0 + t;
    if (ii < ny - pad) {
      s_coef[t] = dt_h * (1.0 / a.celldy[ii]);
      s_ey0[t] = a.edgedy[ii];
      s_ey1[t] = a.edgedy[ii + 1];
    }
  }
  const bool face_ok = jj < nx + 1 - pad;
  const bool cell_ok = (t < kCols - 1) && (jj < nx - pad);
  const bool face_owner = face_ok && (t < kCols - 1);
  double iex = 0.0, cxm = 0.0, cx0 = 0.0, icx = 0.0;
  if (face_ok) {
    iex = 1.0 / a.edgedx[jj];
    cxm = a.celldx[jj - 1];
    cx0 = a.celldx[jj];
    icx = 1.0 / cx0;
  }
  __syncthreads();
  const int i1 = min(i0 + kRows, ny - pad);
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    double F = 0.0, eF = 0.0;
    if (face_ok) {
      const size_t f = fidx(nx, ii, jj);
      const size_t c = cidx(nx, ii, jj);
      mass_energy_flux<false>(a.u[f - 1], a.u[f], a.u[f + 1], s.r_in[c - 2],
                              s.r_in[c - 1], s.r_in[c], s.r_in[c + 1],
                              s.e_in[c - 2], s.e_in[c - 1], s.e_in[c],
                              s.e_in[c + 1], iex, cxm, cx0, icx, s_ey0[k], dt,
                              dt_h, &F, &eF);
      if (face_owner) {
        a.F_x[f] = F;
        mirror_store(a.F_x, nx + 1, ny, pad, ii, jj, F, true, false);
      }
    }
    sF[t] = F;
    seF[t] = eF;
    __syncthreads();
    if (cell_ok) {
      const size_t c = cidx(nx, ii, jj);
      double r_new, e_new;
      mass_energy_update<kFirst>(s.r_in[c], s.e_in[c], a.rho_old[c],
                                 s_coef[k] * icx, s_ey0[k], s_ey1[k], sF[t],
                                 sF[t + 1], seF[t], seF[t + 1], &r_new, &e_new);
      s.r_out[c] = r_new;
      s.e_out[c] = e_new;
      mirror_store(s.r_out, nx, ny, pad, ii, jj, r_new, false, false);
      mirror_store(s.e_out, nx, ny, pad, ii, jj, e_new, false, false);
    }
    __syncthreads();
  }
}

// y sweep: each thread marches down its column; face row ii+1 is computed
// in iteration ii and reused by the cell below.
template <bool kFirst>
__global__ void __launch_bounds__(kCols) k_mass_sweep_y(const StepArgs a,
                                                        const SweepArgs s) {
  __shared__ double s_iey[kRows + 1], s_cy[kRows + 2], s_icy[kRows + 1];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  const double dt = a.ra[kRaDt], dt_h = a.ra[kRaDtH];
  // Face rows i0 .. i0+kRows, cell rows i0-1 .. i0+kRows.
  if (threadIdx.x < kRows + 2) {
    const int ii = i0 - 1 + threadIdx.x;
    if (ii < ny) s_cy[threadIdx.x] = a.celldy[ii];
  }
  if (threadIdx.x < kRows + 1) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      s_iey[threadIdx.x] = 1.0 / a.edgedy[ii];
      s_icy[threadIdx.x] = 1.0 / a.celldy[ii];
    }
  }
  __syncthreads();
  if (jj >= nx - pad) return;
  const double icx = 1.0 / a.celldx[jj];
  const double ex0 = a.edgedx[jj], ex1 = a.edgedx[jj + 1];
  const int i1 = min(i0 + kRows, ny - pad);
  const int last_face = ny - pad;  // the north boundary face row
  // Windows at face row f: cells f-2..f+1, velocities f-1..f+1.
  double r[4], e[4], w[3];
  for (int q = 0; q < 4; ++q) {
    const size_t c = cidx(nx, i0 - 2 + q, jj);
    r[q] = s.r_in[c];
    e[q] = s.e_in[c];
  }
  for (int q = 0; q < 3; ++q) w[q] = a.v[cidx(nx, i0 - 1 + q, jj)];
  double F0, eF0;
  mass_energy_flux<true>(w[0], w[1], w[2], r[0], r[1], r[2], r[3], e[0], e[1],
                         e[2], e[3], s_iey[0], s_cy[0], s_cy[1], s_icy[0], ex0,
                         dt, dt_h, &F0, &eF0);
  {
    const size_t c = cidx(nx, i0, jj);
    a.F_y[c] = F0;
    mirror_store(a.F_y, nx, ny + 1, pad, i0, jj, F0, false, true);
  }
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    // Cell row ii keeps its input values for the update before the window
    // slides to face row ii+1.
    const double r_c = r[2], e_c = e[2];
    for (int q = 0; q < 3; ++q) {
      r[q] = r[q + 1];
      e[q] = e[q + 1];
    }
    const size_t c_next = cidx(nx, ii + 2, jj);
    r[3] = s.r_in[c_next];
    e[3] = s.e_in[c_next];
    w[0] = w[1];
    w[1] = w[2];
    w[2] = a.v[cidx(nx, ii + 2, jj)];
    double F1, eF1;
    mass_energy_flux<true>(w[0], w[1], w[2], r[0], r[1], r[2], r[3], e[0],
                           e[1], e[2], e[3], s_iey[k + 1], s_cy[k + 1],
                           s_cy[k + 2], s_icy[k + 1], ex0, dt, dt_h, &F1, &eF1);
    if (ii + 1 < i1 || ii + 1 == last_face) {
      const size_t c = cidx(nx, ii + 1, jj);
      a.F_y[c] = F1;
      mirror_store(a.F_y, nx, ny + 1, pad, ii + 1, jj, F1, false, true);
    }
    const size_t c = cidx(nx, ii, jj);
    double r_new, e_new;
    mass_energy_update<kFirst>(r_c, e_c, a.rho_old[c], (dt_h * s_icy[k]) * icx,
                               ex0, ex1, F0, F1, eF0, eF1, &r_new, &e_new);
    s.r_out[c] = r_new;
    s.e_out[c] = e_new;
    mirror_store(s.r_out, nx, ny, pad, ii, jj, r_new, false, false);
    mirror_store(s.e_out, nx, ny, pad, ii, jj, e_new, false, false);
    F0 = F1;
    eF0 = eF1;
  }
}

// ===========================================================================
// Advection of momentum (omp3/flow.c:557-970).

// MC-limited upwind value of a velocity at a flux point from its four
// neighbours along the direction (m2, m1 | p0, p1): omp3/flow.c:791-820.
__device__ __forceinline__ double momentum_upwind(double wind, double m2,
                                                  double m1, double p0,
                                                  double p1, double inv_h,
                                                  double d_left, double d_right,
                                                  double dt_h) {
  const bool pos = d_gt0(wind);
  return mc_face(pos, pos ? p0 - m2 : p1 - m1, pos ? m1 - m2 : p0 - m1,
                 pos ? p0 - m1 : p1 - p0, 0.5 * inv_h, 2.0 * inv_h,
                 pos ? m1 : p0, pos ? d_left : d_right, wind * dt_h);
}

// uF_x on interior cells (omp3/flow.c:778-823).
__global__ void __launch_bounds__(kCols) k_flux_uFx(const StepArgs a) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (jj >= nx - pad) return;
  const double dt_h = a.ra[kRaDtH];
  const double iex = 1.0 / a.edgedx[jj];
  const double cxl = a.celldx[jj - 1], cxr = a.celldx[jj];
  const int i1 = min(i0 + kRows, ny - pad);
  for (int ii = i0; ii < i1; ++ii) {
    const size_t f = fidx(nx, ii, jj);
    const double u0 = a.u[f], u1 = a.u[f + 1];
    const double mass = a.edgedy[ii] * 0.5 * (a.F_x[f] + a.F_x[f + 1]);
    const double wind = 0.5 * (u0 + u1);
    const double val = mass * momentum_upwind(wind, a.u[f - 1], u0, u1, a.u[f + 2],
                                              iex, cxl, cxr, dt_h);
    a.uF_x[cidx(nx, ii, jj)] = val;
    mirror_store(a.uF_x, nx, ny, pad, ii, jj, val, false, false);
  }
}

// uF_y on corners (omp3/flow.c:826-874).
__global__ void __launch_bounds__(kCols) k_flux_uFy(const StepArgs a) {
  __shared__ double s_iey[kRows], s_cy[kRows + 1];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (threadIdx.x < kRows + 1) {
    const int ii = i0 - 1 + threadIdx.x;
    if (ii < ny) s_cy[threadIdx.x] = a.celldy[ii];
    if (threadIdx.x >= 1 && ii < ny) s_iey[threadIdx.x - 1] = 1.0 / a.edgedy[ii];
  }
  __syncthreads();
  if (jj >= nx + 1 - pad) return;
  const double dt_h = a.ra[kRaDtH];
  const double ex = a.edgedx[jj];
  const int i1 = min(i0 + kRows, ny + 1 - pad);
  double um2 = a.u[fidx(nx, i0 - 2, jj)];
  double um1 = a.u[fidx(nx, i0 - 1, jj)];
  double u0 = a.u[fidx(nx, i0, jj)];
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    const double up = a.u[fidx(nx, ii + 1, jj)];
    const size_t c = cidx(nx, ii, jj);
    const double mass = ex * 0.5 * (a.F_y[c] + a.F_y[c - 1]);
    const double wind = 0.5 * (a.v[c - 1] + a.v[c]);
    const double val = mass * momentum_upwind(wind, um2, um1, u0, up, s_iey[k],
                                              s_cy[k], s_cy[k + 1], dt_h);
    a.uF_y[fidx(nx, ii, jj)] = val;
    mirror_store(a.uF_y, nx + 1, ny + 1, pad, ii, jj, val, false, false);
    um2 = um1;
    um1 = u0;
    u0 = up;
  }
}

// vF_x on corners (omp3/flow.c:877-925).
__global__ void __launch_bounds__(kCols) k_flux_vFx(const StepArgs a) {
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (jj >= nx + 1 - pad) return;
  const double dt_h = a.ra[kRaDtH];
  const double iex = 1.0 / a.edgedx[jj];
  const double cxl = a.celldx[jj - 1], cxr = a.celldx[jj];
  const int i1 = min(i0 + kRows, ny + 1 - pad);
  double u_dn = a.u[fidx(nx, i0 - 1, jj)], F_dn = a.F_x[fidx(nx, i0 - 1, jj)];
  for (int ii = i0; ii < i1; ++ii) {
    const size_t f = fidx(nx, ii, jj);
    const size_t c = cidx(nx, ii, jj);
    const double u0 = a.u[f], F0 = a.F_x[f];
    const double mass = a.celldy[ii] * 0.5 * (F0 + F_dn);
    const double wind = 0.5 * (u0 + u_dn);
    const double val = mass * momentum_upwind(wind, a.v[c - 2], a.v[c - 1], a.v[c],
                                              a.v[c + 1], iex, cxl, cxr, dt_h);
    a.vF_x[f] = val;
    mirror_store(a.vF_x, nx + 1, ny + 1, pad, ii, jj, val, false, false);
    u_dn = u0;
    F_dn = F0;
  }
}

// vF_y on interior cells (omp3/flow.c:928-970).
__global__ void __launch_bounds__(kCols) k_flux_vFy(const StepArgs a) {
  __shared__ double s_iey[kRows], s_cy[kRows + 1];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  if (threadIdx.x < kRows + 1) {
    const int ii = i0 - 1 + threadIdx.x;
    if (ii < ny) s_cy[threadIdx.x] = a.celldy[ii];
    if (threadIdx.x >= 1 && ii < ny) s_iey[threadIdx.x - 1] = 1.0 / a.edgedy[ii];
  }
  __syncthreads();
  if (jj >= nx - pad) return;
  const double dt_h = a.ra[kRaDtH];
  const double cx = a.celldx[jj];
  const int i1 = min(i0 + kRows, ny - pad);
  double vm = a.v[cidx(nx, i0 - 1, jj)];
  double v0 = a.v[cidx(nx, i0, jj)];
  double vp = a.v[cidx(nx, i0 + 1, jj)];
  double F0 = a.F_y[cidx(nx, i0, jj)];
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    const double vp2 = a.v[cidx(nx, ii + 2, jj)];
    const double F1 = a.F_y[cidx(nx, ii + 1, jj)];
    const double mass = cx * 0.5 * (F0 + F1);
    const double wind = 0.5 * (v0 + vp);
    const double val = mass * momentum_upwind(wind, vm, v0, vp, vp2, s_iey[k],
                                              s_cy[k], s_cy[k + 1], dt_h);
    a.vF_y[cidx(nx, ii, jj)] = val;
    mirror_store(a.vF_y, nx, ny, pad, ii, jj, val, false, false);
    vm = v0;
    v0 = vp;
    vp = vp2;
    F0 = F1;
  }
}

// Momentum updates (omp3/flow.c:577-668, 683-771).  kWhich: 0 rho_u by uF_x,
// 1 rho_u by uF_y, 2 rho_v by vF_x, 3 rho_v by vF_y; kVel recomputes the
// velocity from the post-advection density.
template <int kWhich, bool kVel>
__global__ void __launch_bounds__(kCols) k_momentum_update(const StepArgs a) {
  constexpr bool kU = kWhich < 2;
  __shared__ double s_row[kRows], s_wy0[kRows], s_wy1[kRows];
  const int nx = a.nx, ny = a.ny, pad = a.pad;
  const int jj = pad + blockIdx.x * kCols + threadIdx.x;
  const int i0 = pad + blockIdx.y * kRows;
  const double dt_h = a.ra[kRaDtH];
  if (threadIdx.x < kRows) {
    const int ii = i0 + threadIdx.x;
    if (ii < ny) {
      // Row factor of the flux divergence: 1/celldy for x fluxes of rho_u
      // and rho_v, 1/edgedy for the y fluxes.
      const double h = (kWhich == 0 || kWhich == 2) ? a.celldy[ii] : a.edgedy[ii];
      s_row[threadIdx.x] = dt_h * (1.0 / h);
      if (!kU && kVel) {
        const double ey = a.edgedy[ii];
        s_wy0[threadIdx.x] = a.celldy[ii] / (2.0 * ey);
        s_wy1[threadIdx.x] = a.celldy[ii - 1] / (2.0 * ey);
      }
    }
  }
  __syncthreads();
  const int col_end = kU ? nx + 1 - pad : nx - pad;
  const int row_end = kU ? ny - pad : ny + 1 - pad;
  if (jj >= col_end) return;
  const double hx = (kWhich == 0 || kWhich == 2) ? a.edgedx[jj] : a.celldx[jj];
  const double ihx = 1.0 / hx;
  double wx0 = 0.0, wx1 = 0.0;
  if (kU && kVel) {
    const double ex = a.edgedx[jj];
    wx0 = a.celldx[jj] / (2.0 * ex);
    wx1 = a.celldx[jj - 1] / (2.0 * ex);
  }
  const int i1 = min(i0 + kRows, row_end);
  for (int ii = i0; ii < i1; ++ii) {
    const int k = ii - i0;
    const size_t f = fidx(nx, ii, jj);
    const size_t c = cidx(nx, ii, jj);
    double diff;
    if (kWhich == 0) diff = a.uF_x[c] - a.uF_x[c - 1];
    else if (kWhich == 1) diff = a.uF_y[f + (nx + 1)] - a.uF_y[f];
    else if (kWhich == 2) diff = a.vF_x[f + 1] - a.vF_x[f];
    else diff = a.vF_y[c] - a.vF_y[c - nx];
    double* mom = kU ? a.rho_u + f : a.rho_v + c;
    const double m = fma(-(s_row[k] * ihx), diff, *mom);
    *mom = m;
    if (kVel) {
      double rbar;
      if (kU) rbar = fma(a.rho[c], wx0, a.rho[c - 1] * wx1);
      else rbar = fma(a.rho[c], s_wy0[k], a.rho[c - nx] * s_wy1[k]);
      const double vel = d_is_zero(rbar) ? 0.0 : m * d_rcp(rbar);
      if (kU) {
        a.u[f] = vel;
        mirror_store(a.u, nx + 1, ny, pad, ii, jj, vel, true, false);
      } else {
        a.v[c] = vel;
        mirror_store(a.v, nx, ny + 1, pad, ii, jj, vel, false, true);
      }
    }
  }
}

inline dim3 strip_grid(int cols, int rows, int cols_per_cta = kCols) {
  return dim3((unsigned)((cols + cols_per_cta - 1) / cols_per_cta),
              (unsigned)((rows + kRows - 1) / kRows));
}

template <int W, bool V>
void launch_update(cudaStream_t s, const StepArgs& a) {
  const bool u = W < 2;
  const int cols = u ? (a.nx + 1 - 2 * a.pad) : (a.nx - 2 * a.pad);
  const int rows = u ? (a.ny - 2 * a.pad) : (a.ny + 1 - 2 * a.pad);
  k_momentum_update<W, V><<<strip_grid(cols, rows), kCols, 0, s>>>(a);
}

void launch_mass(cudaStream_t s, const StepArgs& a, bool dir_y, bool first,
                 const SweepArgs& sw) {
  const int pad = a.pad;
  if (dir_y) {
    const dim3 g = strip_grid(a.nx - 2 * pad, a.ny - 2 * pad);
    if (first) k_mass_sweep_y<true><<<g, kCols, 0, s>>>(a, sw);
    else k_mass_sweep_y<false><<<g, kCols, 0, s>>>(a, sw);
  } else {
    // Faces pad .. nx-pad; every CTA advances 127 columns.
    const dim3 g = strip_grid(a.nx + 1 - 2 * pad, a.ny - 2 * pad, kCols - 1);
    if (first) k_mass_sweep_x<true><<<g, kCols, 0, s>>>(a, sw);
    else k_mass_sweep_x<false><<<g, kCols, 0, s>>>(a, sw);
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
  StepArgs a;
  a.nx = mesh->local_nx;
  a.ny = mesh->local_ny;
  a.pad = mesh->pad;
  a.edgedx = mesh->edgedx;
  a.edgedy = mesh->edgedy;
  a.celldx = mesh->celldx;
  a.celldy = mesh->celldy;
  a.P = P; a.rho = rho; a.rho_old = rho_old; a.e = e; a.u = u; a.v = v;
  a.rho_u = rho_u; a.rho_v = rho_v; a.Qxx = Qxx; a.Qyy = Qyy;
  a.F_x = F_x; a.F_y = F_y; a.uF_x = uF_x; a.uF_y = uF_y; a.vF_x = vF_x;
  a.vF_y = vF_y; a.ra = reduce_array;
  a.dt = mesh->dt;
  a.dt_h = mesh->dt_h;
  a.max_dt = mesh->max_dt;
  a.first_step = (tt == 0);
  const int nx = a.nx, ny = a.ny, pad = a.pad;

  StepProfiler prof;
  prof.begin(s);
  // Lagrangian phase.
  prof.mark("lag_pressure");
  k_lag_pressure<<<strip_grid(nx, ny), kCols, 0, s>>>(a);
  prof.mark("lag_viscosity");
  k_lag_viscosity<<<strip_grid(nx - 2 * pad, ny - 2 * pad), kCols, 0, s>>>(a);
  prof.mark("lag_viscous_accel");
  k_lag_viscous_accel<<<strip_grid(nx + 1 - 2 * pad, ny + 1 - 2 * pad), kCols, 0, s>>>(a);
  prof.mark("lag_energy_dt");
  cudaMemsetAsync(reduce_array + kRaTicket, 0, sizeof(double), s);
  cudaMemsetAsync(reduce_array + kRaMinBits, 0xff, sizeof(double), s);
  k_lag_energy_dt<<<strip_grid(nx - 2 * pad, ny - 2 * pad), kCols, 0, s>>>(a);

  // Mass and energy: the first sweep writes into the two cell-sized buffers
  // that hold momentum fluxes later in the step (uF_x, vF_y), the second
  // sweep writes back into rho/e, so neither sweep updates its own input.
  const SweepArgs first{rho, e, uF_x, vF_y};
  const SweepArgs second{uF_x, vF_y, rho, e};
  const bool x_first = (tt % 2 == 0);
  prof.mark(x_first ? "mass_sweep_x" : "mass_sweep_y");
  launch_mass(s, a, !x_first, true, first);
  prof.mark(x_first ? "mass_sweep_y" : "mass_sweep_x");
  launch_mass(s, a, x_first, false, second);

  // Momentum: flux kernel, then update kernel, in the reference order.
  const dim3 g_cell = strip_grid(nx - 2 * pad, ny - 2 * pad);
  const dim3 g_corner = strip_grid(nx + 1 - 2 * pad, ny + 1 - 2 * pad);
  if (tt % 2) {
    prof.mark("flux_uFx");
    k_flux_uFx<<<g_cell, kCols, 0, s>>>(a);
    prof.mark("update_rho_u");
    launch_update<0, true>(s, a);
    prof.mark("flux_uFy");
    k_flux_uFy<<<g_corner, kCols, 0, s>>>(a);
    prof.mark("update_rho_u");
    launch_update<1, false>(s, a);
    prof.mark("flux_vFx");
    k_flux_vFx<<<g_corner, kCols, 0, s>>>(a);
    prof.mark("update_rho_v");
    launch_update<2, true>(s, a);
    prof.mark("flux_vFy");
    k_flux_vFy<<<g_cell, kCols, 0, s>>>(a);
    prof.mark("update_rho_v");
    launch_update<3, false>(s, a);
  } else {
    prof.mark("flux_uFy");
    k_flux_uFy<<<g_corner, kCols, 0, s>>>(a);
    prof.mark("update_rho_u");
    launch_update<1, true>(s, a);
    prof.mark("flux_uFx");
    k_flux_uFx<<<g_cell, kCols, 0, s>>>(a);
    prof.mark("update_rho_u");
    launch_update<0, false>(s, a);
    prof.mark("flux_vFy");
    k_flux_vFy<<<g_cell, kCols, 0, s>>>(a);
    prof.mark("update_rho_v");
    launch_update<3, true>(s, a);
    prof.mark("flux_vFx");
    k_flux_vFx<<<g_corner, kCols, 0, s>>>(a);
    prof.mark("update_rho_v");
    launch_update<2, false>(s, a);
  }
  {
    const int st = check_launch("solve_hydro_2d (fused)");
    if (st != GB300_OK) return st;
  }
  double pair[2];
  cudaMemcpyAsync(pair, reduce_array + kRaDt, sizeof(pair), cudaMemcpyDeviceToHost, s);
  const cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    return record_error(GB300_ERR_CUDA, "solve_hydro_2d (fused): %s", cudaGetErrorString(err));
  }
  prof.end();
  mesh->dt = pair[0];
  mesh->dt_h = pair[1];
  return GB300_OK;
}

}  // namespace flow
