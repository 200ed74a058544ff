/*
 * flow_arch.h -- the single-rank GPU arch layer that the flow host driver
 * needs around the GB300 kernel set (libflow_gb300_arch.so).
 *
 * The reference driver (main.c, flow_data.c) takes these names from the
 * UoB-HPC "arch" project, which flow does not ship.  With a GPU kernel set
 * every array it allocates lives in device memory (cuda/flow.cu passes device
 * pointers to its kernels), so this layer allocates with cudaMalloc, builds
 * the mesh spacing arrays on the host and copies them to the device, and
 * rasterises the params-file problem boxes on the host before uploading them.
 * Each declaration cites the reference call site it serves.
 */
#ifndef FLOW_GB300_ARCH_H
#define FLOW_GB300_ARCH_H

#include <stddef.h>

#include "flow_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MASTER 0
#define MAX_STR_LEN 1024
#define MAX_KEYS 64
#define NO_INVERT 0
#define INVERT_X 1
#define INVERT_Y 2
#define NO_PACK 0
#define PACK 1
#define SEND 0
#define RECV 1

#ifndef TERMINATE
#define TERMINATE(...)                                                        \
  do {                                                                        \
    fprintf(stderr, __VA_ARGS__);                                             \
    exit(EXIT_FAILURE);                                                       \
  } while (0)
#endif

/* Profiling buckets (main.c:123-124); timing is done with CUDA events and
 * ncu instead, so these are no-ops. */
struct Profile {
  int unused;
};
extern struct Profile compute_profile;
extern struct Profile comms_profile;
#define START_PROFILING(profile) ((void)(profile))
#define STOP_PROFILING(profile, name) ((void)(profile), (void)(name))
#define PRINT_PROFILING_RESULTS(profile) ((void)(profile))

/* params file (main.c:20-35, 176-184) */
int get_int_parameter(const char* key, const char* filename);
double get_double_parameter(const char* key, const char* filename);
int get_key_value_parameter(const char* specifier, const char* filename,
                            char* keys, double* values, int* nkeys);
int strmatch(const char* a, const char* b);

/* comms, one rank (main.c:37-39, 117, 166-167) */
void initialise_mpi(int argc, char** argv, int* rank, int* nranks);
void initialise_comms(Mesh* mesh);
void initialise_devices(int rank);
double reduce_all_min(double value);
double reduce_all_sum(double value);
double reduce_to_master(double value);
void barrier(void);

/* memory (flow_data.c:8-15, main.c:149-152): device buffers, zeroed */
size_t allocate_data(double** buf, size_t len);
void deallocate_data(double* buf);
size_t allocate_host_data(double** buf, size_t len);
void deallocate_host_data(double* buf);
void copy_buffer(size_t len, double** src, double** dst, int send);

/* mesh and problem (main.c:40, 52-54, 137-138) */
void initialise_mesh_2d(Mesh* mesh);
void finalise_mesh(Mesh* mesh);
void initialise_shared_data_2d(const int local_nx, const int local_ny,
                               const int pad, const double width,
                               const double height, const char* params_filename,
                               const double* edgex, const double* edgey,
                               SharedData* shared_data);
void finalise_shared_data(SharedData* shared_data);

int within_tolerance(const double expected, const double actual,
                     const double tolerance);

/* VisIt field dump (main.c:108-114, 129-135): <arr_name><tt>.dat (the
 * interior as little-endian doubles, row by row) and <arr_name><tt>.bov (its
 * header), in the working directory.  Asynchronous: the call stages the
 * interior on the device (on the kernel set's stream, gb300_get_stream, in
 * order with the writes of arr) and returns; the host copy runs on a side
 * stream and a writer thread writes the files, so the timestep stream never
 * waits for the host or the disk.  At most two dumps are in flight (a third
 * call waits for the oldest to be written). */
void write_all_ranks_to_visit(const int global_nx, const int global_ny,
                              const int local_nx, const int local_ny,
                              const int pad, const int x_off, const int y_off,
                              const int rank, const int nranks,
                              int* neighbours, double* arr,
                              const char* arr_name, const int tt,
                              const double elapsed_sim_time);
/* Waits until every dump requested so far is on disk (also run at exit). */
void write_all_ranks_flush(void);

#ifdef __cplusplus
}
#endif

#endif /* FLOW_GB300_ARCH_H */
