/*
 * flow_main.c -- C host driver of the GB300 kernel set: the timestep loop of
 * the reference driver (main.c:12-141) with its validation (main.c:144-212),
 * over the GPU arch layer (libflow_gb300_arch.so) and the kernel set
 * (libflow_gb300.so).
 *
 *   flow.gb300 <params file> [--quiet] [--exact]
 *
 * --exact selects the stage-by-stage step (GB300_MODE_EXACT) instead of the
 * fused one.
 *
 * Reads nx, ny, iterations, dt, visit_dump and problem_N boxes from the params
 * file, and width/height/max_dt/sim_end from ../arch.params (defaults 1, 1,
 * 10, 10 when that file is absent).  Prints the per-iteration timestep and
 * conservation totals like the reference, the wallclock of the timed loop
 * (solve_hydro_2d + print_conservation, main.c:80-93), and the validation
 * against flow.tests when it holds an entry for the params file.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime.h>

#include "../../include/flow_arch.h"
#include "../../include/flow_gb300.h"

#define C_T 0.3
#define VALIDATE_TOLERANCE 1.0e-5

static double wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static double arch_param(const char* key, double fallback) {
  FILE* fp = fopen("../arch.params", "r");
  if (!fp) return fallback;
  fclose(fp);
  return get_double_parameter(key, "../arch.params");
}

static void fail_if_error(const char* where) {
  if (gb300_last_error() != GB300_OK) {
    TERMINATE("%s: %s\n", where, gb300_last_error_message());
  }
}

/* Interior totals of density and specific energy, as main.c:154-167 sums
 * them, compared with flow.tests (main.c:173-206). */
static int validate(const int nx, const int ny, const int pad,
                    const char* params, double* density, double* energy) {
  double* hd;
  double* he;
  allocate_host_data(&hd, (size_t)nx * ny);
  allocate_host_data(&he, (size_t)nx * ny);
  copy_buffer((size_t)nx * ny, &density, &hd, RECV);
  copy_buffer((size_t)nx * ny, &energy, &he, RECV);
  double dtot = 0.0, etot = 0.0;
  for (int ii = pad; ii < ny - pad; ++ii) {
    for (int jj = pad; jj < nx - pad; ++jj) {
      dtot += hd[(size_t)ii * nx + jj];
      etot += he[(size_t)ii * nx + jj];
    }
  }
  deallocate_host_data(hd);
  deallocate_host_data(he);
  const char* base = strrchr(params, '/');
  base = base ? base + 1 : params;
  char* keys = (char*)malloc(MAX_KEYS * (MAX_STR_LEN + 1));
  double values[MAX_KEYS];
  int n = 0;
  FILE* fp = fopen("flow.tests", "r");
  const int have = fp != NULL;
  if (fp) fclose(fp);
  if (!have || !get_key_value_parameter(base, "flow.tests", keys, values, &n) || n < 2) {
    printf("Warning. Test entry was not found, could NOT validate.\n");
    printf("density total %.17e, energy total %.17e\n", dtot, etot);
    free(keys);
    return 1;
  }
  const int e_first = strmatch(&keys[0], "energy");
  const double exp_e = e_first ? values[0] : values[1];
  const double exp_d = e_first ? values[1] : values[0];
  free(keys);
  printf("\nExpected energy  %.12e, result was %.12e.\n", exp_e, etot);
  printf("Expected density %.12e, result was %.12e.\n", exp_d, dtot);
  const int pass = within_tolerance(exp_e, etot, VALIDATE_TOLERANCE) &&
                   within_tolerance(exp_d, dtot, VALIDATE_TOLERANCE);
  printf(pass ? "PASSED validation.\n" : "FAILED validation.\n");
  return pass ? 0 : 2;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    TERMINATE("usage: ./flow.gb300 <parameter_filename> [--quiet] [--exact]\n");
  }
  const char* params = argv[1];
  int quiet = 0;
  for (int k = 2; k < argc; ++k) {
    if (strcmp(argv[k], "--quiet") == 0) {
      quiet = 1;
    } else if (strcmp(argv[k], "--exact") == 0) {
      gb300_set_mode(GB300_MODE_EXACT);
    } else {
      TERMINATE("unknown option %s\n", argv[k]);
    }
  }
  gb300_set_verbose(!quiet);

  Mesh mesh;
  memset(&mesh, 0, sizeof(mesh));
  mesh.global_nx = get_int_parameter("nx", params);
  mesh.global_ny = get_int_parameter("ny", params);
  mesh.niters = get_int_parameter("iterations", params);
  mesh.pad = 2;
  mesh.local_nx = mesh.global_nx + 2 * mesh.pad;
  mesh.local_ny = mesh.global_ny + 2 * mesh.pad;
  mesh.width = arch_param("width", 1.0);
  mesh.height = arch_param("height", 1.0);
  mesh.max_dt = arch_param("max_dt", 10.0);
  mesh.sim_end = arch_param("sim_end", 10.0);
  mesh.dt = C_T * get_double_parameter("dt", params);
  mesh.dt_h = mesh.dt;
  const int visit_dump = get_int_parameter("visit_dump", params);

  initialise_mpi(argc, argv, &mesh.rank, &mesh.nranks);
  initialise_comms(&mesh);
  initialise_devices(mesh.rank);
  initialise_mesh_2d(&mesh);

  SharedData sd;
  initialise_shared_data_2d(mesh.local_nx, mesh.local_ny, mesh.pad, mesh.width,
                            mesh.height, params, mesh.edgex, mesh.edgey, &sd);
  handle_boundary_2d(mesh.local_nx, mesh.local_ny, &mesh, sd.density, NO_INVERT, PACK);
  handle_boundary_2d(mesh.local_nx, mesh.local_ny, &mesh, sd.energy, NO_INVERT, PACK);
  fail_if_error("initial ghost fill");

  /* The eight flux/momentum arrays of flow_data.c:8-15. */
  double* mom_x; double* mom_y; double* F_x; double* F_y;
  double* uF_x; double* uF_y; double* vF_x; double* vF_y;
  const size_t nf = (size_t)(mesh.local_nx + 1) * (mesh.local_ny + 1);
  allocate_data(&mom_x, nf); allocate_data(&mom_y, nf);
  allocate_data(&F_x, nf); allocate_data(&F_y, nf);
  allocate_data(&uF_x, nf); allocate_data(&uF_y, nf);
  allocate_data(&vF_x, nf); allocate_data(&vF_y, nf);

  set_timestep(mesh.local_nx, mesh.local_ny, sd.Qxx, sd.Qyy, sd.density,
               sd.energy, &mesh, sd.reduce_array0, 0, mesh.celldx, mesh.celldy);
  fail_if_error("set_timestep");

  printf("Number of ranks: %d\n", mesh.nranks);
  double wallclock = 0.0, elapsed = 0.0;
  for (int tt = 0; tt < mesh.niters; ++tt) {
    if (!quiet) printf("\nIteration %d\n", tt + 1);
    const double w0 = wtime();
    solve_hydro_2d(&mesh, tt, sd.pressure, sd.density, sd.density_old,
                   sd.energy, sd.u, sd.v, mom_x, mom_y, sd.Qxx, sd.Qyy, F_x,
                   F_y, uF_x, uF_y, vF_x, vF_y, sd.reduce_array0);
    print_conservation(mesh.local_nx, mesh.local_ny, sd.density, sd.energy,
                       sd.reduce_array0, &mesh);
    wallclock += wtime() - w0;
    fail_if_error("timestep");
    elapsed += mesh.dt;
    if (elapsed >= mesh.sim_end) {
      printf("reached end of simulation time\n");
      break;
    }
    if (!quiet) {
      printf("Simulation time: %.4lfs\nWallclock:       %.4lfs\n", elapsed, wallclock);
    }
    if (visit_dump) {
      write_all_ranks_to_visit(mesh.global_nx + 2 * mesh.pad, mesh.global_ny + 2 * mesh.pad,
                               mesh.local_nx, mesh.local_ny, mesh.pad, mesh.x_off,
                               mesh.y_off, mesh.rank, mesh.nranks, mesh.neighbours,
                               sd.density, "density", tt, elapsed);
    }
  }
  barrier();
  const int rc = validate(mesh.local_nx, mesh.local_ny, mesh.pad, params, sd.density, sd.energy);
  printf("Wallclock %.4fs, Elapsed Simulation Time %.4fs\n", wallclock, elapsed);

  deallocate_data(mom_x); deallocate_data(mom_y); deallocate_data(F_x);
  deallocate_data(F_y); deallocate_data(uF_x); deallocate_data(uF_y);
  deallocate_data(vF_x); deallocate_data(vF_y);
  finalise_shared_data(&sd);
  finalise_mesh(&mesh);
  return rc == 2 ? 2 : 0;
}
