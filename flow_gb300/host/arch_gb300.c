/*
 * arch_gb300.c -- single-rank GPU arch layer of the flow host driver
 * (include/flow_arch.h): params parsing, device allocation, uniform mesh
 * set-up, problem set-up (the params boxes, rasterised on the device by the
 * kernel set's gb300_fill_boxes) and the VisIt dump.  Compiled into
 * libflow_gb300_arch.so, which links libflow_gb300.so.
 */
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/flow_arch.h"
#include "../../include/flow_gb300.h"

struct Profile compute_profile;
struct Profile comms_profile;

static void cuda_or_die(cudaError_t err, const char* what) {
  if (err != cudaSuccess) {
    TERMINATE("%s failed: %s\n", what, cudaGetErrorString(err));
  }
}

/* ---- params ------------------------------------------------------------- */

/* Finds the line whose first token is `key`; returns the text after it in a
 * static buffer, or NULL. */
static const char* param_line(const char* key, const char* filename) {
  static char line[MAX_STR_LEN];
  FILE* fp = fopen(filename, "r");
  if (!fp) TERMINATE("could not open parameter file %s\n", filename);
  const size_t klen = strlen(key);
  const char* found = NULL;
  while (fgets(line, sizeof(line), fp)) {
    char* p = line;
    while (*p == ' ' || *p == '\t') ++p;
    if (strncmp(p, key, klen) == 0 &&
        (p[klen] == ' ' || p[klen] == '\t' || p[klen] == '\n' ||
         p[klen] == '\r' || p[klen] == '\0')) {
      found = p + klen;
      break;
    }
  }
  fclose(fp);
  return found;
}

int get_int_parameter(const char* key, const char* filename) {
  const char* rest = param_line(key, filename);
  if (!rest) TERMINATE("parameter %s not found in %s\n", key, filename);
  return (int)strtol(rest, NULL, 10);
}

double get_double_parameter(const char* key, const char* filename) {
  const char* rest = param_line(key, filename);
  if (!rest) TERMINATE("parameter %s not found in %s\n", key, filename);
  return strtod(rest, NULL);
}

int get_key_value_parameter(const char* specifier, const char* filename,
                            char* keys, double* values, int* nkeys) {
  *nkeys = 0;
  const char* rest = param_line(specifier, filename);
  if (!rest) return 0;
  char buf[MAX_STR_LEN];
  strncpy(buf, rest, sizeof(buf) - 1);
  buf[sizeof(buf) - 1] = '\0';
  char* save = NULL;
  for (char* tok = strtok_r(buf, " \t\r\n", &save); tok;
       tok = strtok_r(NULL, " \t\r\n", &save)) {
    char* eq = strchr(tok, '=');
    if (!eq || *nkeys >= MAX_KEYS) continue;
    *eq = '\0';
    char* k = &keys[(*nkeys) * (MAX_STR_LEN + 1)];
    strncpy(k, tok, MAX_STR_LEN);
    k[MAX_STR_LEN] = '\0';
    values[*nkeys] = strtod(eq + 1, NULL);
    (*nkeys)++;
  }
  return 1;
}

int strmatch(const char* a, const char* b) { return strcmp(a, b) == 0; }

/* ---- comms (one rank) ----------------------------------------------------- */

void initialise_mpi(int argc, char** argv, int* rank, int* nranks) {
  (void)argc;
  (void)argv;
  *rank = MASTER;
  *nranks = 1;
}

void initialise_comms(Mesh* mesh) {
  for (int k = 0; k < 4; ++k) mesh->neighbours[k] = FLOW_EDGE;
  mesh->x_off = 0;
  mesh->y_off = 0;
}

void initialise_devices(int rank) {
  int count = 0;
  cuda_or_die(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
  if (count == 0) TERMINATE("no CUDA device: the GB300 kernel set has no CPU path\n");
  cuda_or_die(cudaSetDevice(rank % count), "cudaSetDevice");
}

double reduce_all_min(double value) { return value; }
double reduce_all_sum(double value) { return value; }
double reduce_to_master(double value) { return value; }
void barrier(void) { cuda_or_die(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); }

/* ---- memory --------------------------------------------------------------- */

size_t allocate_data(double** buf, size_t len) {
  const size_t bytes = (len ? len : 1) * sizeof(double);
  cuda_or_die(cudaMalloc((void**)buf, bytes), "cudaMalloc");
  cuda_or_die(cudaMemset(*buf, 0, bytes), "cudaMemset");
  return bytes;
}

void deallocate_data(double* buf) { cudaFree(buf); }

size_t allocate_host_data(double** buf, size_t len) {
  *buf = (double*)calloc(len ? len : 1, sizeof(double));
  if (!*buf) TERMINATE("host allocation of %zu doubles failed\n", len);
  return len * sizeof(double);
}

void deallocate_host_data(double* buf) { free(buf); }

void copy_buffer(size_t len, double** src, double** dst, int send) {
  cuda_or_die(cudaMemcpy(*dst, *src, len * sizeof(double),
                         send == SEND ? cudaMemcpyHostToDevice
                                      : cudaMemcpyDeviceToHost),
              "copy_buffer");
}

/* ---- mesh ----------------------------------------------------------------- */

static double* upload(const double* h, size_t n) {
  double* d = NULL;
  cuda_or_die(cudaMalloc((void**)&d, n * sizeof(double)), "cudaMalloc");
  cuda_or_die(cudaMemcpy(d, h, n * sizeof(double), cudaMemcpyHostToDevice),
              "cudaMemcpy");
  return d;
}

void initialise_mesh_2d(Mesh* mesh) {
  const int nx = mesh->local_nx, ny = mesh->local_ny;
  double* ex = (double*)malloc(sizeof(double) * (nx + 1));
  double* ey = (double*)malloc(sizeof(double) * (ny + 1));
  double* dxs = (double*)malloc(sizeof(double) * (nx + 1));
  double* dys = (double*)malloc(sizeof(double) * (ny + 1));
  const double dx = mesh->width / (double)mesh->global_nx;
  const double dy = mesh->height / (double)mesh->global_ny;
  for (int jj = 0; jj <= nx; ++jj) {
    ex[jj] = mesh->width * (double)(mesh->x_off + jj - mesh->pad) / mesh->global_nx;
    dxs[jj] = dx;
  }
  for (int ii = 0; ii <= ny; ++ii) {
    ey[ii] = mesh->height * (double)(mesh->y_off + ii - mesh->pad) / mesh->global_ny;
    dys[ii] = dy;
  }
  mesh->edgex = upload(ex, nx + 1);
  mesh->edgey = upload(ey, ny + 1);
  mesh->edgedx = upload(dxs, nx + 1);
  mesh->celldx = upload(dxs, nx + 1);
  mesh->edgedy = upload(dys, ny + 1);
  mesh->celldy = upload(dys, ny + 1);
  free(ex);
  free(ey);
  free(dxs);
  free(dys);
}

void finalise_mesh(Mesh* mesh) {
  cudaFree(mesh->edgex);
  cudaFree(mesh->edgey);
  cudaFree(mesh->edgedx);
  cudaFree(mesh->edgedy);
  cudaFree(mesh->celldx);
  cudaFree(mesh->celldy);
}

/* The problem boxes of the params file (problem_0, problem_1, ...: density,
 * energy, xpos, ypos, width, height) as rows of 6 doubles; returns the count. */
static int parse_boxes(const char* params, double* boxes, int max_boxes) {
  char* keys = (char*)malloc(MAX_KEYS * (MAX_STR_LEN + 1));
  double values[MAX_KEYS];
  int nb = 0;
  for (int pp = 0;; ++pp) {
    char spec[64];
    snprintf(spec, sizeof(spec), "problem_%d", pp);
    int n = 0;
    if (!get_key_value_parameter(spec, params, keys, values, &n)) break;
    if (nb == max_boxes) TERMINATE("more than %d problem boxes\n", max_boxes);
    double* b = boxes + 6 * nb;
    int have = 0;
    for (int k = 0; k < n; ++k) {
      const char* key = &keys[k * (MAX_STR_LEN + 1)];
      if (strmatch(key, "density")) { b[0] = values[k]; have |= 1; }
      else if (strmatch(key, "energy")) { b[1] = values[k]; have |= 2; }
      else if (strmatch(key, "xpos")) { b[2] = values[k]; have |= 4; }
      else if (strmatch(key, "ypos")) { b[3] = values[k]; have |= 8; }
      else if (strmatch(key, "width")) { b[4] = values[k]; have |= 16; }
      else if (strmatch(key, "height")) { b[5] = values[k]; have |= 32; }
    }
    if (have != 63) TERMINATE("%s needs density energy xpos ypos width height\n", spec);
    ++nb;
  }
  free(keys);
  return nb;
}

void initialise_shared_data_2d(const int local_nx, const int local_ny,
                               const int pad, const double width,
                               const double height, const char* params_filename,
                               const double* edgex, const double* edgey,
                               SharedData* sd) {
  (void)pad;
  (void)width;
  (void)height;
  const size_t nc = (size_t)local_nx * local_ny;
  const size_t nf = (size_t)(local_nx + 1) * (local_ny + 1);
  allocate_data(&sd->pressure, nc);
  allocate_data(&sd->density, nc);
  allocate_data(&sd->density_old, nc);
  allocate_data(&sd->energy, nc);
  allocate_data(&sd->u, nf);
  allocate_data(&sd->v, nf);
  allocate_data(&sd->Qxx, nc);
  allocate_data(&sd->Qyy, nc);
  allocate_data(&sd->reduce_array0, nc);
  allocate_data(&sd->reduce_array1, nc);
  if (!edgex || !edgey) TERMINATE("initialise_mesh_2d must run first\n");
  /* The boxes are rasterised on the device (gb300_fill_boxes): no host
   * arrays and no copies of the fields. */
  double boxes[6 * GB300_MAX_BOXES];
  const int nb = parse_boxes(params_filename, boxes, GB300_MAX_BOXES);
  if (gb300_fill_boxes(local_nx, local_ny, edgex, edgey, boxes, nb, sd->density,
                       sd->energy) != GB300_OK) {
    TERMINATE("problem set-up: %s\n", gb300_last_error_message());
  }
  cuda_or_die(cudaDeviceSynchronize(), "problem set-up");
}

void finalise_shared_data(SharedData* sd) {
  deallocate_data(sd->pressure);
  deallocate_data(sd->density);
  deallocate_data(sd->density_old);
  deallocate_data(sd->energy);
  deallocate_data(sd->u);
  deallocate_data(sd->v);
  deallocate_data(sd->Qxx);
  deallocate_data(sd->Qyy);
  deallocate_data(sd->reduce_array0);
  deallocate_data(sd->reduce_array1);
}

int within_tolerance(const double expected, const double actual,
                     const double tolerance) {
  const double scale = expected != 0.0 ? (expected > 0 ? expected : -expected) : 1.0;
  const double d = actual - expected;
  return (d < 0 ? -d : d) <= tolerance * scale;
}

void write_all_ranks_to_visit(const int global_nx, const int global_ny,
                              const int local_nx, const int local_ny,
                              const int pad, const int x_off, const int y_off,
                              const int rank, const int nranks,
                              int* neighbours, double* arr,
                              const char* arr_name, const int tt,
                              const double elapsed_sim_time) {
  (void)global_nx; (void)global_ny; (void)x_off; (void)y_off; (void)nranks;
  (void)neighbours;
  if (rank != MASTER) return;
  const size_t n = (size_t)local_nx * local_ny;
  double* h = (double*)malloc(n * sizeof(double));
  cuda_or_die(cudaMemcpy(h, arr, n * sizeof(double), cudaMemcpyDeviceToHost), "visit dump");
  char name[256];
  snprintf(name, sizeof(name), "%s%d.dat", arr_name, tt);
  FILE* fp = fopen(name, "wb");
  if (fp) {
    for (int ii = pad; ii < local_ny - pad; ++ii) {
      fwrite(&h[(size_t)ii * local_nx + pad], sizeof(double), (size_t)(local_nx - 2 * pad), fp);
    }
    fclose(fp);
  }
  snprintf(name, sizeof(name), "%s%d.bov", arr_name, tt);
  fp = fopen(name, "w");
  if (fp) {
    fprintf(fp, "TIME: %.12e\nDATA_FILE: %s%d.dat\nDATA_SIZE: %d %d 1\n"
                "DATA_FORMAT: DOUBLE\nVARIABLE: %s\nDATA_ENDIAN: LITTLE\n"
                "CENTERING: zonal\nBRICK_ORIGIN: 0. 0. 0.\nBRICK_SIZE: %d %d 1\n",
            elapsed_sim_time, arr_name, tt, local_nx - 2 * pad,
            local_ny - 2 * pad, arr_name, local_nx - 2 * pad, local_ny - 2 * pad);
    fclose(fp);
  }
  free(h);
}
