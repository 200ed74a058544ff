/*
 * arch_shim.h -- ORACLE TEST INFRASTRUCTURE.  A CPU restatement of the parts
 * of the UoB-HPC "arch" layer that the flow mini-app needs.
 *
 * The reference sources include ../shared.h, ../mesh.h, ../shared_data.h,
 * ../comms.h and ../params.h from arch (flow_interface.h:2-4, main.c:1-4,
 * omp3/flow.c:2-3, omp3/flow.h:1), and arch is not shipped with flow.  This
 * header supplies every arch name those files use, written from how the flow
 * sources call them:
 *   - params:   get_int_parameter / get_double_parameter (main.c:20-35),
 *               get_key_value_parameter + strmatch (main.c:176-184),
 *               MAX_KEYS / MAX_STR_LEN (main.c:174)
 *   - mesh:     initialise_mesh_2d (main.c:40), handle_boundary_2d with
 *               NO_INVERT / INVERT_X / INVERT_Y and PACK (omp3/flow.c:156-157)
 *   - data:     initialise_shared_data_2d (main.c:52-54), allocate_data
 *               (flow_data.c:8-15), copy_buffer(..., RECV) (main.c:151-152)
 *   - comms:    initialise_mpi/comms/devices (main.c:37-39), reduce_all_min
 *               (omp3/flow.c:100), reduce_to_master (omp3/flow.c:988-989),
 *               reduce_all_sum (main.c:166-167), barrier (main.c:117)
 *   - helpers:  min, minmod (omp3/flow.c:94, 177, 353), within_tolerance
 *               (main.c:197), TERMINATE, MASTER, profiling macros
 *               (omp3/flow.c:57,69; main.c:123-124), VisIt writer (main.c:109)
 * Only the single-rank, no-MPI behaviour is provided (Makefile:2-4 default).
 *
 * Only tests, the smoke check and the CPU baseline of the benchmark use this.
 */
#ifndef FLOW_ORACLE_ARCH_SHIM_H
#define FLOW_ORACLE_ARCH_SHIM_H

#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/flow_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MASTER 0
#define MAX_STR_LEN 1024
#define MAX_KEYS 64

/* handle_boundary_2d modes */
#define NO_INVERT 0
#define INVERT_X 1
#define INVERT_Y 2
#define NO_PACK 0
#define PACK 1

/* copy_buffer directions */
#define SEND 0
#define RECV 1

#define TERMINATE(...)                                                        \
  do {                                                                        \
    fprintf(stderr, __VA_ARGS__);                                             \
    exit(EXIT_FAILURE);                                                       \
  } while (0)

/* Profiling is compiled out unless ENABLE_PROFILING is given (Makefile:6),
 * which this shim does not support. */
struct Profile {
  int unused;
};
extern struct Profile compute_profile;
extern struct Profile comms_profile;
#define START_PROFILING(profile) ((void)(profile))
#define STOP_PROFILING(profile, name) ((void)(profile), (void)(name))
#define PRINT_PROFILING_RESULTS(profile) ((void)(profile))

/* Under nvcc (the reference's cuda set, built with cuda/shared.h) CUDA's own
 * min overloads and the device minmod of cuda/shared.h take their place. */
#ifndef __CUDACC__
/* Ordinary minimum: the first argument when it is strictly smaller. */
static inline double min(const double a, const double b) {
  return (a < b) ? a : b;
}

/* Slope limiter: zero unless both arguments are non-zero with the same sign,
 * otherwise the argument of smaller magnitude (the second one on a tie). */
static inline double minmod(const double a, const double b) {
  if ((a > 0.0 && b > 0.0) || (a < 0.0 && b < 0.0)) {
    return (fabs(a) < fabs(b)) ? a : b;
  }
  return 0.0;
}
#endif

/* --- params --------------------------------------------------------------- */
int get_int_parameter(const char* key, const char* filename);
double get_double_parameter(const char* key, const char* filename);
/* Finds the line whose first token is `specifier` and parses its key=value
 * tokens.  keys[i*(MAX_STR_LEN+1)] holds the i-th key.  Returns 0 when the
 * specifier is absent. */
int get_key_value_parameter(const char* specifier, const char* filename,
                            char* keys, double* values, int* nkeys);
int strmatch(const char* a, const char* b);

/* --- comms (single rank) -------------------------------------------------- */
void initialise_mpi(int argc, char** argv, int* rank, int* nranks);
void initialise_comms(Mesh* mesh);
void initialise_devices(int rank);
/* Transport hooks of a decomposed run (tests only): fill the ghost layers of
 * arr (nx x ny) facing other ranks; replace *value by its minimum over the
 * ranks. */
typedef int (*flow_shim_halo_fn)(void* ctx, const Mesh* mesh, double* arr, int nx, int ny,
                                 int invert);
typedef int (*flow_shim_min_fn)(void* ctx, double* value);
void flow_shim_set_halo(flow_shim_halo_fn fn, void* ctx);
void flow_shim_set_reduce_min(flow_shim_min_fn fn, void* ctx);
double reduce_all_min(double value);
double reduce_all_sum(double value);
double reduce_to_master(double value);
void barrier(void);
void finalise_comms(void);

/* --- memory --------------------------------------------------------------- */
size_t allocate_data(double** buf, size_t len);
void deallocate_data(double* buf);
size_t allocate_host_data(double** buf, size_t len);
void deallocate_host_data(double* buf);
void copy_buffer(size_t len, double** src, double** dst, int send);

/* --- mesh and problem set-up ---------------------------------------------- */
void initialise_mesh_2d(Mesh* mesh);
void finalise_mesh(Mesh* mesh);
void initialise_shared_data_2d(const int local_nx, const int local_ny,
                               const int pad, const double width,
                               const double height, const char* params_filename,
                               const double* edgex, const double* edgey,
                               SharedData* shared_data);
void finalise_shared_data(SharedData* shared_data);

/* Rasterises the `problem_N` boxes of a params file into density/energy:
 * a cell takes a box's values when its left/bottom edge coordinate lies in
 * [pos, pos+extent).  Later boxes overwrite earlier ones. */
void set_problem_2d(const int local_nx, const int local_ny,
                    const char* params_filename, const double* edgex,
                    const double* edgey, double* density, double* energy);

/* Reflective ghost fill of one array of nx x ny points (pad ghost layers on
 * each side), see arch_shim.c. */
void handle_boundary_2d(const int nx, const int ny, Mesh* mesh, double* arr,
                        const int invert, const int pack);

int within_tolerance(const double expected, const double actual,
                     const double tolerance);

void write_all_ranks_to_visit(const int global_nx, const int global_ny,
                              const int local_nx, const int local_ny,
                              const int pad, const int x_off, const int y_off,
                              const int rank, const int nranks,
                              int* neighbours, double* arr,
                              const char* arr_name, const int tt,
                              const double elapsed_sim_time);

#ifdef __cplusplus
}
#endif

#endif /* FLOW_ORACLE_ARCH_SHIM_H */
