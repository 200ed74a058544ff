/*
 * flow_mesh.h -- host-side mesh and state descriptors shared by the GB300
 * kernel set, its host driver and the CPU oracle.
 *
 * The flow mini-app takes its Mesh and SharedData structs from the UoB-HPC
 * "arch" layer, which is not part of the flow repository.  The kernel-set ABI
 * (flow_interface.h:16-30 of the reference) passes a `Mesh*` into every
 * timestep call, so a drop-in kernel set needs the struct definition.  The
 * fields below are exactly the ones the reference reads or writes:
 *   main.c:18-40           global/local sizes, pad, width/height, max_dt,
 *                          sim_end, dt, dt_h, rank, nranks, niters
 *   main.c:109-113         x_off, y_off, neighbours (field dumps)
 *   omp3/flow.c:22-51      edgedx/edgedy/celldx/celldy, dt, dt_h, pad, rank
 *   omp3/flow.c:103-105    set_timestep writes dt and dt_h
 *   main.c:52-54           edgex/edgey feed the problem rasteriser
 *
 * Conventions (all sizes are in cells):
 *   local_nx = global_nx + 2*pad (one rank), pad = 2.
 *   Cell arrays are local_ny rows x local_nx columns, row-major, index
 *   ii*local_nx + jj.  x-face arrays are local_ny x (local_nx+1); y-face
 *   arrays use row stride local_nx with local_ny+1 rows (omp3/flow.c:129);
 *   corner arrays are (local_ny+1) x (local_nx+1).
 *   The spacing arrays hold local_n+1 entries.  For a GPU kernel set they are
 *   device pointers; dt and dt_h are always host doubles.
 */
#ifndef FLOW_GB300_MESH_H
#define FLOW_GB300_MESH_H

/* A build inside the arch project can use arch's own Mesh/SharedData: define
 * FLOW_EXTERNAL_MESH_HEADER (e.g. "../mesh.h") when compiling the kernel set.
 * The kernel set only reads the fields listed above by name. */
enum { FLOW_NORTH = 0, FLOW_EAST = 1, FLOW_SOUTH = 2, FLOW_WEST = 3 };
#define FLOW_EDGE (-1) /* neighbour value at a physical (reflective) wall */

#ifdef FLOW_EXTERNAL_MESH_HEADER
#include FLOW_EXTERNAL_MESH_HEADER
#else

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int global_nx, global_ny; /* interior cells of the whole problem */
  int local_nx, local_ny;   /* padded cells held by this rank */
  int pad;                  /* ghost layers on each side (2) */
  int x_off, y_off;         /* offset of this rank's first interior cell */
  int rank, nranks;
  int niters;
  int neighbours[4];        /* FLOW_EDGE or a rank, ordered N,E,S,W */
  double width, height;     /* physical extent of the global domain */
  double max_dt;            /* start value of the CFL minimum */
  double sim_end;           /* simulated time at which the driver stops */
  double dt, dt_h;          /* full and half timestep (host scalars) */
  double* edgex;            /* x position of face jj (left edge of cell jj) */
  double* edgey;
  double* edgedx;           /* face-centred spacing */
  double* edgedy;
  double* celldx;           /* cell widths */
  double* celldy;
} Mesh;

/* Cell- and face-centred state owned by the host driver (arch SharedData). */
typedef struct {
  double* pressure;
  double* density;
  double* density_old;
  double* energy;
  double* u;
  double* v;
  double* Qxx;
  double* Qyy;
  double* reduce_array0;
  double* reduce_array1;
} SharedData;

#ifdef __cplusplus
}
#endif

#endif /* FLOW_EXTERNAL_MESH_HEADER */

#endif /* FLOW_GB300_MESH_H */
