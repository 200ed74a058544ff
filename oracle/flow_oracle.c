/*
 * flow_oracle.c -- ORACLE TEST INFRASTRUCTURE.  A plain-C restatement of the
 * reference omp3 kernel set (omp3/flow.c) for the flow timestep, used only by
 * the tests, the smoke check and the CPU-baseline leg of the benchmark as the
 * checker of the GB300 kernels.  It exports the same entry points as
 * flow_interface.h:16-30 and omp3/flow.h:4-88, so it is itself a drop-in
 * kernel set for the reference's host driver.
 *
 * Arithmetic is written in the reference's evaluation order (left to right,
 * no reassociation) so that, built with -ffp-contract=off, it reproduces the
 * reference bit for bit; oracle/Makefile builds the reference itself next to
 * it and the tests compare the two.  The arch helpers it needs (min, minmod,
 * handle_boundary_2d, reductions) come from oracle/arch/arch_shim.c.
 *
 * Differences from the reference that do not change any field value:
 *   - printing is off unless flow_oracle_verbose is set (the reference prints
 *     dt and conservation totals every step, omp3/flow.c:18-20, 991-994);
 *   - conservation sums are accumulated per row and then over rows in a fixed
 *     order, so they do not depend on the thread count.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "arch/arch_shim.h"

/* Constants of flow_interface.h:7-9 and flow_data.h:5. */
#define ORC_GAM 1.4
#define ORC_C_Q 3.0
#define ORC_C_T 0.3
#define ORC_C_M (1.5 / ORC_C_T)

int flow_oracle_verbose = 0;

/* Index helpers.  nx is the padded cell count in x.  Cell and y-face arrays
 * share row stride nx; x-face and corner arrays use nx+1. */
#define CSTR ((size_t)nx)
#define FSTR ((size_t)nx + 1)
#define AT_C(a, ii, jj) (a)[(size_t)(ii) * CSTR + (size_t)(jj)]
#define AT_F(a, ii, jj) (a)[(size_t)(ii) * FSTR + (size_t)(jj)]

/* ------------------------------------------------------------------------ */
/* equation_of_state, omp3/flow.c:55-70: P = (gamma-1) rho e on every cell.  */
void equation_of_state(const int nx, const int ny, double* P, const double* rho,
                       const double* e) {
#pragma omp parallel for
  for (int ii = 0; ii < ny; ++ii) {
    for (int jj = 0; jj < nx; ++jj) {
      AT_C(P, ii, jj) = (ORC_GAM - 1.0) * AT_C(rho, ii, jj) * AT_C(e, ii, jj);
    }
  }
}

/* set_timestep, omp3/flow.c:73-106: CFL minimum over the interior starting
 * from max_dt, then the leapfrog update of dt and dt_h. */
void set_timestep(const int nx, const int ny, double* Qxx, double* Qyy,
                  const double* rho, const double* e, Mesh* mesh,
                  double* reduce_array, const int first_step,
                  const double* celldx, const double* celldy) {
  (void)reduce_array;
  const int pad = mesh->pad;
  double dt_min = mesh->max_dt;
#pragma omp parallel for reduction(min : dt_min)
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      const double sound = sqrt(ORC_GAM * (ORC_GAM - 1.0) * AT_C(e, ii, jj));
      const double cfl_x =
          celldx[jj] / sqrt(sound * sound +
                            2.0 * AT_C(Qxx, ii, jj) / AT_C(rho, ii, jj));
      const double cfl_y =
          celldy[ii] / sqrt(sound * sound +
                            2.0 * AT_C(Qyy, ii, jj) / AT_C(rho, ii, jj));
      const double cell_min = min(cfl_x, cfl_y);
      dt_min = min(dt_min, cell_min);
    }
  }
  const double global_min = reduce_all_min(dt_min);
  const double limited = min(global_min, ORC_C_M * mesh->dt_h);
  mesh->dt = 0.5 * (ORC_C_T * limited + mesh->dt_h);
  mesh->dt_h = first_step ? mesh->dt : ORC_C_T * limited;
}

/* Volume-weighted density on x-face (ii,jj) and y-face (ii,jj),
 * omp3/flow.c:134-141. */
static inline double rho_on_xface(const int nx, const double* rho,
                                  const double* edgedx, const double* celldx,
                                  const double* celldy, int ii, int jj) {
  return (AT_C(rho, ii, jj) * celldx[jj] * celldy[ii] +
          AT_C(rho, ii, jj - 1) * celldx[jj - 1] * celldy[ii]) /
         (2.0 * edgedx[jj] * celldy[ii]);
}
static inline double rho_on_yface(const int nx, const double* rho,
                                  const double* edgedy, const double* celldx,
                                  const double* celldy, int ii, int jj) {
  return (AT_C(rho, ii, jj) * celldx[jj] * celldy[ii] +
          AT_C(rho, ii - 1, jj) * celldx[jj] * celldy[ii - 1]) /
         (2.0 * celldx[jj] * edgedy[ii]);
}

/* pressure_acceleration, omp3/flow.c:110-158.  Note the y momentum and
 * velocity use the cell row stride nx (omp3/flow.c:129,148). */
void pressure_acceleration(const int nx, const int ny, Mesh* mesh,
                           const double dt, double* rho_u, double* rho_v,
                           double* u, double* v, const double* P,
                           const double* rho, const double* edgedx,
                           const double* edgedy, const double* celldx,
                           const double* celldy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      AT_F(rho_u, ii, jj) -=
          dt * (AT_C(P, ii, jj) - AT_C(P, ii, jj - 1)) / edgedx[jj];
      AT_C(rho_v, ii, jj) -=
          dt * (AT_C(P, ii, jj) - AT_C(P, ii - 1, jj)) / edgedy[ii];
      const double rx = rho_on_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
      const double ry = rho_on_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
      AT_F(u, ii, jj) = (rx == 0.0) ? 0.0 : AT_F(rho_u, ii, jj) / rx;
      AT_C(v, ii, jj) = (ry == 0.0) ? 0.0 : AT_C(rho_v, ii, jj) / ry;
    }
  }
  handle_boundary_2d(nx + 1, ny, mesh, u, INVERT_X, PACK);
  handle_boundary_2d(nx, ny + 1, mesh, v, INVERT_Y, PACK);
}

/* Limited compressive velocity jumps of the artificial viscosity,
 * omp3/flow.c:177-198: `lo`, `mid`, `hi`, `hi2` are the four velocities
 * at offsets -1, 0, +1, +2 along the direction. */
static inline void viscous_jumps(double lo, double mid, double hi, double hi2,
                                 double* jump, double* curv) {
  *jump = min(0.0, hi - mid);
  *curv = 0.5 * (fabs(min(0.0, (hi2 - hi)) - min(0.0, (hi - mid))) +
                 fabs(min(0.0, (hi - mid)) - min(0.0, (mid - lo))));
}

/* artificial_viscosity, omp3/flow.c:160-245. */
void artificial_viscosity(const int nx, const int ny, Mesh* mesh,
                          const double dt, double* Qxx, double* Qyy, double* u,
                          double* v, double* rho_u, double* rho_v,
                          const double* rho, const double* edgedx,
                          const double* edgedy, const double* celldx,
                          const double* celldy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      double u_i, u_ii, v_i, v_ii;
      viscous_jumps(AT_F(u, ii, jj - 1), AT_F(u, ii, jj), AT_F(u, ii, jj + 1),
                    AT_F(u, ii, jj + 2), &u_i, &u_ii);
      viscous_jumps(AT_C(v, ii - 1, jj), AT_C(v, ii, jj), AT_C(v, ii + 1, jj),
                    AT_C(v, ii + 2, jj), &v_i, &v_ii);
      AT_C(Qxx, ii, jj) = -ORC_C_Q * AT_C(rho, ii, jj) * u_i * u_ii;
      AT_C(Qyy, ii, jj) = -ORC_C_Q * AT_C(rho, ii, jj) * v_i * v_ii;
    }
  }
  handle_boundary_2d(nx, ny, mesh, Qxx, NO_INVERT, PACK);
  handle_boundary_2d(nx, ny, mesh, Qyy, NO_INVERT, PACK);

#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      AT_F(rho_u, ii, jj) -=
          dt * (AT_C(Qxx, ii, jj) - AT_C(Qxx, ii, jj - 1)) / celldx[jj];
      AT_C(rho_v, ii, jj) -=
          dt * (AT_C(Qyy, ii, jj) - AT_C(Qyy, ii - 1, jj)) / celldy[ii];
      const double rx = rho_on_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
      const double ry = rho_on_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
      AT_F(u, ii, jj) = (rx == 0.0) ? 0.0 : AT_F(rho_u, ii, jj) / rx;
      AT_C(v, ii, jj) = (ry == 0.0) ? 0.0 : AT_C(rho_v, ii, jj) / ry;
    }
  }
  handle_boundary_2d(nx + 1, ny, mesh, u, INVERT_X, PACK);
  handle_boundary_2d(nx, ny + 1, mesh, v, INVERT_Y, PACK);
}

/* shock_heating_and_work, omp3/flow.c:248-290. */
void shock_heating_and_work(const int nx, const int ny, Mesh* mesh,
                            const double dt_h, double* e, const double* P,
                            const double* u, const double* v, const double* rho,
                            const double* Qxx, const double* Qyy,
                            const double* celldx, const double* celldy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      const double r = AT_C(rho, ii, jj);
      const double p = AT_C(P, ii, jj);
      const double dudx = (AT_F(u, ii, jj + 1) - AT_F(u, ii, jj)) / celldx[jj];
      const double dvdy = (AT_C(v, ii + 1, jj) - AT_C(v, ii, jj)) / celldy[ii];
      const double div_dt = (dudx + dvdy) * dt_h;
      const double e_q =
          AT_C(e, ii, jj) -
          dt_h * (AT_C(Qxx, ii, jj) * dudx + AT_C(Qyy, ii, jj) * dvdy) / r;
      const double rho_c = r / (1.0 + div_dt);
      const double e_c = e_q - (p * div_dt) / r;
      const double work =
          0.5 * div_dt * (p + (ORC_GAM - 1.0) * e_c * rho_c) / r;
      AT_C(e, ii, jj) = (r == 0.0) ? 0.0 : e_q - work;
    }
  }
  handle_boundary_2d(nx, ny, mesh, e, NO_INVERT, PACK);
}

/* Mass and energy sweep along x, omp3/flow.c:326-439. */
void x_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* u, double* F_x, double* eF_x,
                            const double* celldx, const double* edgedx,
                            const double* celldy, const double* edgedy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      const double invdx = 1.0 / edgedx[jj];
      const double um = AT_F(u, ii, jj - 1);
      const double u0 = AT_F(u, ii, jj);
      const double up = AT_F(u, ii, jj + 1);
      const double s_c = 0.5 * invdx * (up - um);
      const double s_r = 2.0 * invdx * (u0 - um);
      const double s_l = 2.0 * invdx * (up - u0);
      const double u_tc = u0 - 0.5 * u0 * dt * minmod(s_c, minmod(s_r, s_l));

      const double r_m2 = AT_C(rho, ii, jj - 2);
      const double r_m1 = AT_C(rho, ii, jj - 1);
      const double r_0 = AT_C(rho, ii, jj);
      const double r_p1 = AT_C(rho, ii, jj + 1);
      double limiter = 0.0;
      const double rho_jump = (r_0 - r_m1);
      if (rho_jump) {
        const double smooth =
            (u_tc >= 0.0) ? (r_m1 - r_m2) / rho_jump : (r_p1 - r_0) / rho_jump;
        limiter = (smooth + fabs(smooth)) / (1.0 + fabs(smooth));
      }
      const double rho_up = (u_tc >= 0.0) ? r_m1 : r_0;
      const double flux =
          (u_tc * rho_up + 0.5 * fabs(u_tc) *
                               (1.0 - fabs((u_tc * dt_h) / celldx[jj])) *
                               limiter * rho_jump);
      AT_F(F_x, ii, jj) = flux;

      const double e_m2 = AT_C(e, ii, jj - 2);
      const double e_m1 = AT_C(e, ii, jj - 1);
      const double e_0 = AT_C(e, ii, jj);
      const double e_p1 = AT_C(e, ii, jj + 1);
      const double a0 = 0.5 * invdx * (e_0 - e_m2);
      const double b0 = 2.0 * invdx * (e_m1 - e_m2);
      const double c0 = 2.0 * invdx * (e_0 - e_m1);
      const double a1 = 0.5 * invdx * (e_p1 - e_m1);
      const double b1 = 2.0 * invdx * (e_0 - e_m1);
      const double c1 = 2.0 * invdx * (e_p1 - e_0);
      const double e_face =
          (u_tc > 0.0)
              ? e_m1 + 0.5 * minmod(minmod(a0, b0), c0) *
                           (celldx[jj - 1] - u_tc * dt_h)
              : e_0 - 0.5 * minmod(minmod(a1, b1), c1) *
                          (celldx[jj] + u_tc * dt_h);
      AT_F(eF_x, ii, jj) = edgedy[ii] * e_face * AT_F(F_x, ii, jj);
    }
  }
  handle_boundary_2d(nx + 1, ny, mesh, F_x, INVERT_X, PACK);

#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      AT_C(rho, ii, jj) -= dt_h *
                           (edgedy[ii + 1] * AT_F(F_x, ii, jj + 1) -
                            edgedy[ii] * AT_F(F_x, ii, jj)) /
                           (celldx[jj] * celldy[ii]);
      const double rho_e =
          (AT_C(rho_old, ii, jj) * AT_C(e, ii, jj) -
           (dt_h * (AT_F(eF_x, ii, jj + 1) - AT_F(eF_x, ii, jj))) /
               (celldx[jj] * celldy[ii]));
      const double denom = first ? AT_C(rho_old, ii, jj) : AT_C(rho, ii, jj);
      AT_C(e, ii, jj) = (denom == 0.0) ? 0.0 : rho_e / denom;
    }
  }
  handle_boundary_2d(nx, ny, mesh, rho, NO_INVERT, PACK);
  handle_boundary_2d(nx, ny, mesh, e, NO_INVERT, PACK);
}

/* Mass and energy sweep along y, omp3/flow.c:442-554.  The Van Leer
 * smoothness direction follows the sign of v itself, not of the
 * half-step velocity (omp3/flow.c:477). */
void y_mass_and_energy_flux(const int nx, const int ny, const int first,
                            Mesh* mesh, const double dt, const double dt_h,
                            double* rho, double* rho_old, double* e,
                            const double* v, double* F_y, double* eF_y,
                            const double* celldx, const double* edgedx,
                            const double* celldy, const double* edgedy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      const double invdy = 1.0 / edgedy[ii];
      const double vm = AT_C(v, ii - 1, jj);
      const double v0 = AT_C(v, ii, jj);
      const double vp = AT_C(v, ii + 1, jj);
      const double s_c = 0.5 * invdy * (vp - vm);
      const double s_r = 2.0 * invdy * (v0 - vm);
      const double s_l = 2.0 * invdy * (vp - v0);
      const double v_tc = v0 - 0.5 * v0 * dt * minmod(s_c, minmod(s_r, s_l));

      const double r_m2 = AT_C(rho, ii - 2, jj);
      const double r_m1 = AT_C(rho, ii - 1, jj);
      const double r_0 = AT_C(rho, ii, jj);
      const double r_p1 = AT_C(rho, ii + 1, jj);
      const double rho_jump = (r_0 - r_m1);
      double limiter = 0.0;
      if (rho_jump) {
        const double smooth =
            (v0 >= 0.0) ? (r_m1 - r_m2) / rho_jump : (r_p1 - r_0) / rho_jump;
        limiter = (smooth + fabs(smooth)) / (1.0 + fabs(smooth));
      }
      const double rho_up = (v_tc >= 0.0) ? r_m1 : r_0;
      const double flux =
          (v_tc * rho_up + 0.5 * fabs(v_tc) *
                               (1.0 - fabs((v_tc * dt_h) / celldy[ii])) *
                               limiter * rho_jump);
      AT_C(F_y, ii, jj) = flux;

      const double e_m2 = AT_C(e, ii - 2, jj);
      const double e_m1 = AT_C(e, ii - 1, jj);
      const double e_0 = AT_C(e, ii, jj);
      const double e_p1 = AT_C(e, ii + 1, jj);
      const double a0 = 0.5 * invdy * (e_0 - e_m2);
      const double b0 = 2.0 * invdy * (e_m1 - e_m2);
      const double c0 = 2.0 * invdy * (e_0 - e_m1);
      const double a1 = 0.5 * invdy * (e_p1 - e_m1);
      const double b1 = 2.0 * invdy * (e_0 - e_m1);
      const double c1 = 2.0 * invdy * (e_p1 - e_0);
      const double e_face =
          (v_tc > 0.0)
              ? e_m1 + 0.5 * minmod(minmod(a0, b0), c0) *
                           (celldy[ii - 1] - v_tc * dt_h)
              : e_0 - 0.5 * minmod(minmod(a1, b1), c1) *
                          (celldy[ii] + v_tc * dt_h);
      AT_C(eF_y, ii, jj) = edgedx[jj] * e_face * AT_C(F_y, ii, jj);
    }
  }
  handle_boundary_2d(nx, ny + 1, mesh, F_y, INVERT_Y, PACK);

#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      AT_C(rho, ii, jj) -= dt_h *
                           (edgedx[jj + 1] * AT_C(F_y, ii + 1, jj) -
                            edgedx[jj] * AT_C(F_y, ii, jj)) /
                           (celldx[jj] * celldy[ii]);
      const double rho_e =
          (AT_C(rho_old, ii, jj) * AT_C(e, ii, jj) -
           (dt_h * (AT_C(eF_y, ii + 1, jj) - AT_C(eF_y, ii, jj))) /
               (celldx[jj] * celldy[ii]));
      const double denom = first ? AT_C(rho_old, ii, jj) : AT_C(rho, ii, jj);
      AT_C(e, ii, jj) = (denom == 0.0) ? 0.0 : rho_e / denom;
    }
  }
  handle_boundary_2d(nx, ny, mesh, rho, NO_INVERT, PACK);
  handle_boundary_2d(nx, ny, mesh, e, NO_INVERT, PACK);
}

/* advect_mass_and_energy, omp3/flow.c:293-323: x then y on even steps,
 * y then x on odd steps; the first sweep divides by the old density. */
void advect_mass_and_energy(const int nx, const int ny, Mesh* mesh,
                            const int tt, const double dt, const double dt_h,
                            double* rho, double* e, double* rho_old,
                            double* F_x, double* F_y, double* eF_x,
                            double* eF_y, const double* u, const double* v,
                            const double* edgedx, const double* edgedy,
                            const double* celldx, const double* celldy) {
  memcpy(rho_old, rho, sizeof(double) * (size_t)nx * ny);
  if (tt % 2 == 0) {
    x_mass_and_energy_flux(nx, ny, 1, mesh, dt, dt_h, rho, rho_old, e, u, F_x,
                           eF_x, celldx, edgedx, celldy, edgedy);
    y_mass_and_energy_flux(nx, ny, 0, mesh, dt, dt_h, rho, rho_old, e, v, F_y,
                           eF_y, celldx, edgedx, celldy, edgedy);
  } else {
    y_mass_and_energy_flux(nx, ny, 1, mesh, dt, dt_h, rho, rho_old, e, v, F_y,
                           eF_y, celldx, edgedx, celldy, edgedy);
    x_mass_and_energy_flux(nx, ny, 0, mesh, dt, dt_h, rho, rho_old, e, u, F_x,
                           eF_x, celldx, edgedx, celldy, edgedy);
  }
}

/* MC-limited upwind interpolation used by the four momentum fluxes: the
 * value reconstructed at the flux point from the left (`lm`, with slopes
 * of m2,m1,p0) or from the right (`rp`, with slopes of m1,p0,p1). */
static inline double mc_upwind(double wind, double m2, double m1, double p0,
                               double p1, double invd, double d_left,
                               double d_right, double dt_h, double lm,
                               double rp) {
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

/* momentum_x_flux_in_x, omp3/flow.c:778-823: cell-centred flux of rho u. */
void momentum_x_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* u, double* uF_x,
                          const double* F_x, const double* edgedx,
                          const double* edgedy, const double* celldx) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      const double invdx = 1.0 / edgedx[jj];
      const double um = AT_F(u, ii, jj - 1);
      const double u0 = AT_F(u, ii, jj);
      const double up = AT_F(u, ii, jj + 1);
      const double up2 = AT_F(u, ii, jj + 2);
      const double u_cell = 0.5 * (u0 + up);
      const double mass =
          edgedy[ii] * 0.5 * (AT_F(F_x, ii, jj) + AT_F(F_x, ii, jj + 1));
      const double u_up = mc_upwind(u_cell, um, u0, up, up2, invdx,
                                    celldx[jj - 1], celldx[jj], dt_h, u0, up);
      AT_C(uF_x, ii, jj) = mass * u_up;
    }
  }
}

/* momentum_x_flux_in_y, omp3/flow.c:826-874: corner flux of rho u in y. */
void momentum_x_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* u, double* v,
                          double* uF_y, const double* F_y,
                          const double* edgedx, const double* edgedy,
                          const double* celldy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      const double invdy = 1.0 / edgedy[ii];
      const double um2 = AT_F(u, ii - 2, jj);
      const double um1 = AT_F(u, ii - 1, jj);
      const double u0 = AT_F(u, ii, jj);
      const double up = AT_F(u, ii + 1, jj);
      const double v_corner = 0.5 * (AT_C(v, ii, jj - 1) + AT_C(v, ii, jj));
      const double mass =
          edgedx[jj] * 0.5 * (AT_C(F_y, ii, jj) + AT_C(F_y, ii, jj - 1));
      const double u_up = mc_upwind(v_corner, um2, um1, u0, up, invdy,
                                    celldy[ii - 1], celldy[ii], dt_h, um1, u0);
      AT_F(uF_y, ii, jj) = mass * u_up;
    }
  }
}

/* momentum_y_flux_in_x, omp3/flow.c:877-925: corner flux of rho v in x. */
void momentum_y_flux_in_x(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, const double* u, double* v,
                          double* vF_x, const double* F_x,
                          const double* edgedx, const double* celldy,
                          const double* celldx) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      const double invdx = 1.0 / edgedx[jj];
      const double vm2 = AT_C(v, ii, jj - 2);
      const double vm1 = AT_C(v, ii, jj - 1);
      const double v0 = AT_C(v, ii, jj);
      const double vp = AT_C(v, ii, jj + 1);
      const double mass =
          celldy[ii] * 0.5 * (AT_F(F_x, ii, jj) + AT_F(F_x, ii - 1, jj));
      const double u_corner = 0.5 * (AT_F(u, ii, jj) + AT_F(u, ii - 1, jj));
      const double v_up = mc_upwind(u_corner, vm2, vm1, v0, vp, invdx,
                                    celldx[jj - 1], celldx[jj], dt_h, vm1, v0);
      AT_F(vF_x, ii, jj) = mass * v_up;
    }
  }
}

/* momentum_y_flux_in_y, omp3/flow.c:928-970: cell-centred flux of rho v. */
void momentum_y_flux_in_y(const int nx, const int ny, Mesh* mesh,
                          const double dt_h, double* v, double* vF_y,
                          const double* F_y, const double* edgedy,
                          const double* celldx, const double* celldy) {
  const int pad = mesh->pad;
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      const double invdy = 1.0 / edgedy[ii];
      const double vm = AT_C(v, ii - 1, jj);
      const double v0 = AT_C(v, ii, jj);
      const double vp = AT_C(v, ii + 1, jj);
      const double vp2 = AT_C(v, ii + 2, jj);
      const double mass =
          celldx[jj] * 0.5 * (AT_C(F_y, ii, jj) + AT_C(F_y, ii + 1, jj));
      const double v_cell = 0.5 * (v0 + vp);
      const double v_up = mc_upwind(v_cell, vm, v0, vp, vp2, invdy,
                                    celldy[ii - 1], celldy[ii], dt_h, v0, vp);
      AT_C(vF_y, ii, jj) = mass * v_up;
    }
  }
}

/* The four momentum update loops of advect_momentum, omp3/flow.c:577-668. */
static void update_rho_u_by_uF_x(const int nx, const int ny, const int pad,
                                 const double dt_h, double* rho_u, double* u,
                                 const double* uF_x, const double* rho,
                                 const double* edgedx, const double* celldx,
                                 const double* celldy, const int with_u) {
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      AT_F(rho_u, ii, jj) -= dt_h *
                             (AT_C(uF_x, ii, jj) - AT_C(uF_x, ii, jj - 1)) /
                             (edgedx[jj] * celldy[ii]);
      if (with_u) {
        const double rx =
            rho_on_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
        AT_F(u, ii, jj) = (rx == 0.0) ? 0.0 : AT_F(rho_u, ii, jj) / rx;
      }
    }
  }
}

static void update_rho_u_by_uF_y(const int nx, const int ny, const int pad,
                                 const double dt_h, double* rho_u, double* u,
                                 const double* uF_y, const double* rho,
                                 const double* edgedx, const double* edgedy,
                                 const double* celldx, const double* celldy,
                                 const int with_u) {
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < (nx + 1) - pad; ++jj) {
      AT_F(rho_u, ii, jj) -= dt_h *
                             (AT_F(uF_y, ii + 1, jj) - AT_F(uF_y, ii, jj)) /
                             (celldx[jj] * edgedy[ii]);
      if (with_u) {
        const double rx =
            rho_on_xface(nx, rho, edgedx, celldx, celldy, ii, jj);
        AT_F(u, ii, jj) = (rx == 0.0) ? 0.0 : AT_F(rho_u, ii, jj) / rx;
      }
    }
  }
}

static void update_rho_v_by_vF_x(const int nx, const int ny, const int pad,
                                 const double dt_h, double* rho_v, double* v,
                                 const double* vF_x, const double* rho,
                                 const double* edgedx, const double* edgedy,
                                 const double* celldx, const double* celldy,
                                 const int with_v) {
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      AT_C(rho_v, ii, jj) -= dt_h *
                             (AT_F(vF_x, ii, jj + 1) - AT_F(vF_x, ii, jj)) /
                             (edgedx[jj] * celldy[ii]);
      if (with_v) {
        const double ry =
            rho_on_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
        AT_C(v, ii, jj) = (ry == 0.0) ? 0.0 : AT_C(rho_v, ii, jj) / ry;
      }
    }
  }
}

static void update_rho_v_by_vF_y(const int nx, const int ny, const int pad,
                                 const double dt_h, double* rho_v, double* v,
                                 const double* vF_y, const double* rho,
                                 const double* edgedy, const double* celldx,
                                 const double* celldy, const int with_v) {
#pragma omp parallel for
  for (int ii = pad; ii < (ny + 1) - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      AT_C(rho_v, ii, jj) -= dt_h *
                             (AT_C(vF_y, ii, jj) - AT_C(vF_y, ii - 1, jj)) /
                             (celldx[jj] * edgedy[ii]);
      if (with_v) {
        const double ry =
            rho_on_yface(nx, rho, edgedy, celldx, celldy, ii, jj);
        AT_C(v, ii, jj) = (ry == 0.0) ? 0.0 : AT_C(rho_v, ii, jj) / ry;
      }
    }
  }
}

/* advect_momentum, omp3/flow.c:557-775.  Odd steps: x-flux of rho u (with
 * u), y-flux of rho u, x-flux of rho v (with v), y-flux of rho v.  Even
 * steps: y-flux of rho u (with u), x-flux of rho u, y-flux of rho v (with v),
 * x-flux of rho v. */
void advect_momentum(const int nx, const int ny, const int tt, Mesh* mesh,
                     const double dt_h, const double dt, double* u, double* v,
                     double* uF_x, double* uF_y, double* vF_x, double* vF_y,
                     double* rho_u, double* rho_v, const double* rho,
                     const double* F_x, const double* F_y,
                     const double* edgedx, const double* edgedy,
                     const double* celldx, const double* celldy) {
  (void)dt;
  const int pad = mesh->pad;
  if (tt % 2) {
    momentum_x_flux_in_x(nx, ny, mesh, dt_h, u, uF_x, F_x, edgedx, edgedy,
                         celldx);
    handle_boundary_2d(nx, ny, mesh, uF_x, NO_INVERT, PACK);
    update_rho_u_by_uF_x(nx, ny, pad, dt_h, rho_u, u, uF_x, rho, edgedx,
                         celldx, celldy, 1);
    handle_boundary_2d(nx + 1, ny, mesh, u, INVERT_X, PACK);

    momentum_x_flux_in_y(nx, ny, mesh, dt_h, u, v, uF_y, F_y, edgedx, edgedy,
                         celldy);
    handle_boundary_2d(nx + 1, ny + 1, mesh, uF_y, NO_INVERT, PACK);
    update_rho_u_by_uF_y(nx, ny, pad, dt_h, rho_u, u, uF_y, rho, edgedx,
                         edgedy, celldx, celldy, 0);

    momentum_y_flux_in_x(nx, ny, mesh, dt_h, u, v, vF_x, F_x, edgedx, celldy,
                         celldx);
    handle_boundary_2d(nx + 1, ny + 1, mesh, vF_x, NO_INVERT, PACK);
    update_rho_v_by_vF_x(nx, ny, pad, dt_h, rho_v, v, vF_x, rho, edgedx,
                         edgedy, celldx, celldy, 1);
    handle_boundary_2d(nx, ny + 1, mesh, v, INVERT_Y, PACK);

    momentum_y_flux_in_y(nx, ny, mesh, dt_h, v, vF_y, F_y, edgedy, celldx,
                         celldy);
    handle_boundary_2d(nx, ny, mesh, vF_y, NO_INVERT, PACK);
    update_rho_v_by_vF_y(nx, ny, pad, dt_h, rho_v, v, vF_y, rho, edgedy,
                         celldx, celldy, 0);
  } else {
    momentum_x_flux_in_y(nx, ny, mesh, dt_h, u, v, uF_y, F_y, edgedx, edgedy,
                         celldy);
    handle_boundary_2d(nx + 1, ny + 1, mesh, uF_y, NO_INVERT, PACK);
    update_rho_u_by_uF_y(nx, ny, pad, dt_h, rho_u, u, uF_y, rho, edgedx,
                         edgedy, celldx, celldy, 1);
    handle_boundary_2d(nx + 1, ny, mesh, u, INVERT_X, PACK);

    momentum_x_flux_in_x(nx, ny, mesh, dt_h, u, uF_x, F_x, edgedx, edgedy,
                         celldx);
    handle_boundary_2d(nx, ny, mesh, uF_x, NO_INVERT, PACK);
    update_rho_u_by_uF_x(nx, ny, pad, dt_h, rho_u, u, uF_x, rho, edgedx,
                         celldx, celldy, 0);

    momentum_y_flux_in_y(nx, ny, mesh, dt_h, v, vF_y, F_y, edgedy, celldx,
                         celldy);
    handle_boundary_2d(nx, ny, mesh, vF_y, NO_INVERT, PACK);
    update_rho_v_by_vF_y(nx, ny, pad, dt_h, rho_v, v, vF_y, rho, edgedy,
                         celldx, celldy, 1);
    handle_boundary_2d(nx, ny + 1, mesh, v, INVERT_Y, PACK);

    momentum_y_flux_in_x(nx, ny, mesh, dt_h, u, v, vF_x, F_x, edgedx, celldy,
                         celldx);
    handle_boundary_2d(nx + 1, ny + 1, mesh, vF_x, NO_INVERT, PACK);
    update_rho_v_by_vF_x(nx, ny, pad, dt_h, rho_v, v, vF_x, rho, edgedx,
                         edgedy, celldx, celldy, 0);
  }
}

/* solve_hydro_2d, omp3/flow.c:10-52: one full timestep. */
void solve_hydro_2d(Mesh* mesh, int tt, double* P, double* rho,
                    double* rho_old, double* e, double* u, double* v,
                    double* rho_u, double* rho_v, double* Qxx, double* Qyy,
                    double* F_x, double* F_y, double* uF_x, double* uF_y,
                    double* vF_x, double* vF_y, double* reduce_array) {
  const int nx = mesh->local_nx;
  const int ny = mesh->local_ny;
  if (flow_oracle_verbose && mesh->rank == MASTER) {
    printf("Timestep:        %.12e\n", mesh->dt);
  }
  equation_of_state(nx, ny, P, rho, e);
  pressure_acceleration(nx, ny, mesh, mesh->dt, rho_u, rho_v, u, v, P, rho,
                        mesh->edgedx, mesh->edgedy, mesh->celldx,
                        mesh->celldy);
  artificial_viscosity(nx, ny, mesh, mesh->dt, Qxx, Qyy, u, v, rho_u, rho_v,
                       rho, mesh->edgedx, mesh->edgedy, mesh->celldx,
                       mesh->celldy);
  shock_heating_and_work(nx, ny, mesh, mesh->dt_h, e, P, u, v, rho, Qxx, Qyy,
                         mesh->celldx, mesh->celldy);
  set_timestep(nx, ny, Qxx, Qyy, rho, e, mesh, reduce_array, tt == 0,
               mesh->celldx, mesh->celldy);
  /* The energy fluxes reuse the x/y momentum-flux buffers, as the reference
   * does (omp3/flow.c:41-45). */
  advect_mass_and_energy(nx, ny, mesh, tt, mesh->dt, mesh->dt_h, rho, e,
                         rho_old, F_x, F_y, uF_x, uF_y, u, v, mesh->edgedx,
                         mesh->edgedy, mesh->celldx, mesh->celldy);
  advect_momentum(nx, ny, tt, mesh, mesh->dt_h, mesh->dt, u, v, uF_x, uF_y,
                  vF_x, vF_y, rho_u, rho_v, rho, F_x, F_y, mesh->edgedx,
                  mesh->edgedy, mesh->celldx, mesh->celldy);
}

/* Interior totals of rho and rho*e (omp3/flow.c:973-995) in a fixed order:
 * out[0] = mass, out[1] = energy. */
void flow_oracle_conservation(const int nx, const int ny, const int pad,
                              const double* rho, const double* e,
                              double* out) {
  const int rows = ny - 2 * pad;
  double* part = (double*)calloc((size_t)(rows > 0 ? rows : 1) * 2,
                                 sizeof(double));
#pragma omp parallel for
  for (int ii = pad; ii < ny - pad; ++ii) {
    double m = 0.0, en = 0.0;
    for (int jj = pad; jj < nx - pad; ++jj) {
      m += AT_C(rho, ii, jj);
      en += AT_C(rho, ii, jj) * AT_C(e, ii, jj);
    }
    part[2 * (ii - pad)] = m;
    part[2 * (ii - pad) + 1] = en;
  }
  double m = 0.0, en = 0.0;
  for (int rr = 0; rr < rows; ++rr) {
    m += part[2 * rr];
    en += part[2 * rr + 1];
  }
  free(part);
  out[0] = m;
  out[1] = en;
}

/* print_conservation, omp3/flow.c:973-995. */
void print_conservation(const int nx, const int ny, double* rho, double* e,
                        double* reduce_array, Mesh* mesh) {
  (void)reduce_array;
  double tot[2];
  flow_oracle_conservation(nx, ny, mesh->pad, rho, e, tot);
  const double mass = reduce_to_master(tot[0]);
  const double energy = reduce_to_master(tot[1]);
  if (flow_oracle_verbose && mesh->rank == MASTER) {
    printf("Total mass:      %.12e\n", mass);
    printf("Total energy:    %.12e\n", energy);
  }
}
